// learn.cu - training and inference kernels of the learned parts (FP16
// tensor-core MLPs with FP32 accumulation) and their C ABI.
//
// Training step of a batch of `rows` samples (rows a multiple of 16):
//   k_mlp_train_tc  forward, per-row loss gradient dY, backward and the weight
//                   gradients of 128-row tiles, fused, on tcgen05 with tensor-
//                   memory accumulators (at most one CTA per SM; each adds its
//                   weight-gradient sums to the f32 gradient);
//   k_adam          Adam on f32 master weights, refreshing the f16 copy and
//                   the training kernel's swizzled weight image.
//   k_mlp_infer_tc  the forward pass alone, on tcgen05, many tiles per CTA;
//                   for the cache it encodes the queries itself and adds
//                   throughput x radiance to the pixel sums (no input or
//                   output matrix in memory).
// Shapes are template parameters: <IN, NH, OUT> with hidden width 64.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <utility>
#include <vector>

#include "../../include/tpt.h"
#include "arena.h"
#include "mlp.cuh"
#include "tc05.cuh"

namespace tpt {
namespace mlp {

// ------------------------------------------------------------ losses ----
// Each loss writes dL/dy for one row (already multiplied by `scale`, the
// loss scale over the batch size) and returns the row's loss.
// Every loss also has preload(row): the row's loss inputs, read when the
// tile starts so their latency overlaps the forward pass (passed to grad).
struct LossGiven {  // dY supplied by the caller (tests)
  const float *dy;
  float scale;
  static constexpr bool kEncodes = false;
  using Pre = int;
  __device__ Pre preload(int) const { return 0; }
  template <int OUT>
  __device__ float grad(int row, const float *y, float *dy_out, Pre) const {
    for (int o = 0; o < OUT; o++) dy_out[o] = dy[(size_t)row * OUT + o] * scale;
    return 0.f;
  }
};

// ------------------------------------------- fused training (tcgen05) ---
// One training step of a batch on the 5th-generation tensor cores: every CTA
// (one warpgroup, 128 threads; thread t owns row t of the tile and tensor-
// memory lane t) takes 128-row tiles of the batch and runs, per tile,
//   forward   Z_l = H_l W_l^T  (tcgen05.mma, M = 128, f32 in tensor memory);
//             ReLU and f16 rounding in registers, H_{l+1} back to shared memory
//   loss      dY of the tile's rows from the f32 outputs (one row per thread)
//   backward  dH_l = dZ_l W_l (M = 128), masked by H_l > 0 into dZ_{l-1};
//             dW_l += dZ_l^T H_l (M = 64: the layer's outputs, zero-padded;
//             N = its inputs; K = the tile's rows), accumulated over all of
//             the CTA's tiles in tensor memory.
// The MMAs read the swizzled shared-memory tiles of tc05.cuh: the forward
// tiles (X, H_l, W_l) serve K-major in the forward pass and, through MN-major
// descriptors, as the transposed operands of the backward pass and of the
// weight gradients, so nothing is transposed or written to HBM between the
// passes.  A fifth warp issues the MMAs (one thread); completions arrive on
// mbarriers the four rows warps wait on (with a time limit).  The weight-
// gradient MMAs of layer l + 1 are issued after dH_l, so they run off the
// critical path while the rows warps form dZ_{l-1}; dZ_l rotates through
// three shared-memory tiles (l mod 3) so that neither pass overwrites a tile
// an MMA in flight still reads.  The weights arrive by one bulk copy of the
// network's pre-swizzled weight image (written by the Adam step); at the end
// each CTA stages its dW sums in shared memory and adds them to the gradient
// with coalesced vector reductions.
template <int IN, int NH, int OUT>
struct TrainLayout {
  static_assert(IN % 16 == 0 && IN <= 128 && OUT % 16 == 0 && OUT <= 64 && NH >= 1, "supported shapes");
  static constexpr int KB0 = (IN + 63) / 64;  // 64-column blocks of the input tile
  __host__ __device__ static constexpr int in_(int l) { return l == 0 ? IN : HID; }
  __host__ __device__ static constexpr int out_(int l) { return l == NH ? OUT : HID; }
  __host__ __device__ static constexpr uint32_t w_off(int l) {  // weight tile of layer l: its input blocks of out_(l) rows
    uint32_t o = 0;
    for (int j = 0; j < l; j++) o += (uint32_t)((in_(j) + 63) / 64) * out_(j) * 128;
    return o;
  }
  static constexpr uint32_t W_BYTES = w_off(NH + 1);  // the weight image
  static constexpr uint32_t X_OFF = W_BYTES;
  static constexpr uint32_t H_OFF = X_OFF + KB0 * 16384;  // H_1 .. H_NH
  static constexpr uint32_t DZ_OFF = H_OFF + NH * 16384;  // three rotating dZ tiles: dZ_l in tile l % 3
  static constexpr uint32_t BAR_OFF = DZ_OFF + 3 * 16384;
  static constexpr uint32_t SMEM = BAR_OFF + 64 + 1024;  // + slack for the 1024-byte alignment
  __host__ __device__ static constexpr int dw_col(int l) {  // tensor-memory column of layer l's weight gradient
    int c = 64;                         // columns 0..63: the forward / backward accumulator
    for (int j = 0; j < l; j++) c += in_(j);
    return c;
  }
  static constexpr uint32_t TMEM_COLS = 512;
  static_assert(X_OFF % 1024 == 0 && W_BYTES % 16 == 0, "operand tiles start on 1024-byte boundaries");
  static_assert(dw_col(NH + 1) <= (int)TMEM_COLS, "tensor memory");
  static_assert(SMEM <= 227 * 1024, "shared memory");
};

// Byte offset of weight p (layer-major, [out][in] per layer) in the weight
// image: layer l's tile at TrainLayout::w_off(l), its 64-input blocks of
// out rows one after the other, each row 128-byte swizzled.
__host__ __device__ inline uint32_t wimg_offset(const Net &n, int p) {
  int l = 0, off = 0;
  uint32_t img = 0;
  for (;;) {
    const int K = layer_in(n, l), N = layer_out(n, l);
    if (p < off + N * K || l == n_layers(n) - 1) break;
    off += N * K;
    img += (uint32_t)((K + 63) / 64) * N * 128;
    l++;
  }
  const int K = layer_in(n, l), N = layer_out(n, l), q = p - off, o = q / K, i = q - o * K;
  return img + (uint32_t)(i / 64) * N * 128 + tc05::sw128(o, i % 64);
}
__host__ __device__ inline uint32_t wimg_bytes(const Net &n) {
  uint32_t img = 0;
  for (int l = 0; l < n_layers(n); l++) img += (uint32_t)((layer_in(n, l) + 63) / 64) * layer_out(n, l) * 128;
  return img;
}

// ~2 s at 2 GHz: an MMA completion that has not arrived by then never will
constexpr long long TC_WAIT_LIMIT = 4000000000LL;

// Position of float4 i4 of row o in the staged weight-gradient sums: XOR
// swizzled by o mod 8 within each full group of 8 float4, so the 16 rows a
// warp stores at once fall into different banks.
__device__ __forceinline__ int stage_slot(int o, int i4, int k4) {
  return i4 < (k4 & ~7) ? (i4 ^ (o & 7)) : i4;
}

constexpr int TC_THREADS = 160;  // warps 0-3: rows / tensor-memory lanes; warp 4: issues the MMAs

template <int IN, int NH, int OUT, class Loss>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_mlp_train_tc(Net n, const uint8_t *__restrict__ wimg, const __half *__restrict__ X, int rows, Loss loss,
                   float *loss_sum, float *loss_next, int *err) {
  using T = TrainLayout<IN, NH, OUT>;
  using namespace tc05;
  static_assert(T::BAR_OFF - T::H_OFF >= (uint32_t)((IN * HID + (NH - 1) * HID * HID + HID * OUT) * 4),
                "the weight-gradient sums are staged where H and dZ lived");
  extern __shared__ uint8_t tc_raw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + T::BAR_OFF + 32);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const bool rows_warp = warp < 4;           // epilogue: thread t owns row t and lane t
  const bool issuer = warp == 4 && lane == 0;  // the one thread that issues MMAs
  const uint32_t base = smem_addr(sm);
  // barA: forward and dH MMAs; barW[p]: the weight-gradient MMAs of the
  // layers l with l & 1 == p (each has at most one phase outstanding when it
  // is waited on); barL: the weight image
  const uint32_t barA = base + T::BAR_OFF, barW0 = barA + 8, barL = barA + 24;
  uint32_t phA = 0, phW0 = 0, phW1 = 0;
  bool ok = true;

  // the weight image: one bulk copy (in 16 KB pieces) completing on barL.
  // Padding columns of the tiles (past IN) are never read: the forward MMAs
  // stop at K = IN and the weight-gradient MMAs at N = IN.
  // Launched as a chained step, this prologue and the first tile's rows run
  // while the previous step's Adam kernel finishes: the weight image, the
  // gradient and the loss sums are touched only after griddep_wait.
  if (t == 0) griddep_launch();
  if (issuer) {
    bar_init(barA, 1);
    bar_init(barW0, 1);
    bar_init(barW0 + 8, 1);
    bar_init(barL, 1);
    griddep_wait();
    if (loss_next && blockIdx.x == 0) *loss_next = 0.f;  // the next step's loss sum
    bar_expect_bytes(barL, T::W_BYTES);
    for (uint32_t o = 0; o < T::W_BYTES; o += 16384)
      bulk_copy(base + o, wimg + o, T::W_BYTES - o < 16384 ? T::W_BYTES - o : 16384, barL);
  }
  if (warp == 0) tmem_alloc(tslot, T::TMEM_COLS);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tm = *tslot;
  const uint32_t lane_base = tm + ((uint32_t)((warp & 3) * 32) << 16);
  bool weights = false;  // the issuer has seen the weight image arrive
  // descriptors of the tiles' first bytes; a K step adds an offset
  const uint64_t dX = desc(base + T::X_OFF, 16, 1024), dXmn = desc(base + T::X_OFF, 16384, 1024);
  const uint64_t dW = desc(base, 16, 1024), dWmn = desc(base, 16384, 1024);
  const uint64_t dH = desc(base + T::H_OFF, 16, 1024), dHmn = desc(base + T::H_OFF, 16384, 1024);
  const uint64_t dZ = desc(base + T::DZ_OFF, 16, 1024), dZmn = desc(base + T::DZ_OFF, 16384, 1024);
  float lsum = 0.f;
  bool first = true;
  const int n_tiles = (rows + 127) / 128;
  // a rows warp waits for an MMA completion; the whole warp agrees on the
  // outcome (its tensor-memory loads are warp-collective)
  auto wait_rows = [&](uint32_t bar, uint32_t &ph) {
    const bool got = __all_sync(0xffffffffu, bar_wait(bar, ph, TC_WAIT_LIMIT));
    ph ^= 1;
    ok = ok && got;
    return got;
  };

  for (int tile = blockIdx.x; ok && tile < n_tiles; tile += gridDim.x) {
    const int r0 = tile * 128;
    typename Loss::Pre pre{};
    if (rows_warp) {
      if constexpr (Loss::kEncodes) {  // the loss builds its input row t itself (row past the batch: zeros)
        pre = loss.encode(r0 + t, r0 + t < rows, sm + T::X_OFF, t);
      } else {
        if (r0 + t < rows) pre = loss.preload(r0 + t);
        // ---- the input tile (rows past the batch are zero-filled)
        constexpr int CH = IN / 8;
        for (int c = t; c < 128 * CH; c += 128) {
          const int r = c / CH, k8 = c - r * CH;
          const bool in = r0 + r < rows;
          cp_async16(sm + T::X_OFF + (uint32_t)(k8 / 8) * 16384 + sw128_chunk(r, k8 % 8),
                     X + (size_t)(in ? r0 + r : 0) * IN + k8 * 8, in ? 16 : 0);
        }
        cp_async_wait_all();
      }
      fence_async_smem();
      if (first) griddep_wait();  // before this thread's tensor memory, gradient and loss writes
    }
    if (issuer && !weights) weights = ok = bar_wait(barL, 0, TC_WAIT_LIMIT);  // overlapped with the first tile's copies
    if (!(ok = __syncthreads_and(ok))) break;  // every thread leaves together
    // ---- forward (loops rolled: each CTA runs its body for a tile or two,
    // so a compact body keeps instruction fetch off the critical path)
#pragma unroll 1
    for (int l = 0; l <= NH; l++) {
      if (issuer) {
        fence_after();
        const uint64_t a0 = l == 0 ? dX : desc_add(dH, (uint32_t)(l - 1) * 16384);
        const uint64_t b0 = desc_add(dW, T::w_off(l));
        const uint32_t id = idesc_f16(128, T::out_(l), false, false);
        const uint32_t bstride = T::out_(l) * 128;  // between the weight tile's 64-input blocks
#pragma unroll 1
        for (int s = 0; s < T::in_(l) / 16; s++)
          mma_f16(tm, desc_add(a0, (uint32_t)(s >> 2) * 16384 + (uint32_t)(s & 3) * 32),
                  desc_add(b0, (uint32_t)(s >> 2) * bstride + (uint32_t)(s & 3) * 32), id, s > 0);
        commit(barA);
      }
      if (rows_warp && wait_rows(barA, phA)) {
        fence_after();
        float v[64];
        tmem_ld64(lane_base, v);
        if (l < NH) {  // ReLU, f16: row t of H_{l+1}
          uint8_t *dst = sm + T::H_OFF + (uint32_t)l * 16384;
#pragma unroll
          for (int c = 0; c < 8; c++) {
            uint4 q;
            q.x = pack2(fmaxf(v[8 * c], 0.f), fmaxf(v[8 * c + 1], 0.f));
            q.y = pack2(fmaxf(v[8 * c + 2], 0.f), fmaxf(v[8 * c + 3], 0.f));
            q.z = pack2(fmaxf(v[8 * c + 4], 0.f), fmaxf(v[8 * c + 5], 0.f));
            q.w = pack2(fmaxf(v[8 * c + 6], 0.f), fmaxf(v[8 * c + 7], 0.f));
            *reinterpret_cast<uint4 *>(dst + sw128_chunk(t, c)) = q;
          }
        } else {  // the loss of row t; dZ of the output layer (zero past OUT and past the batch)
          uint8_t *dst = sm + T::DZ_OFF + (uint32_t)(NH % 3) * 16384;
          float dy[OUT];
          if (r0 + t < rows) {
            lsum += loss.template grad<OUT>(r0 + t, v, dy, pre);
          } else {
#pragma unroll
            for (int o = 0; o < OUT; o++) dy[o] = 0.f;
          }
#pragma unroll
          for (int c = 0; c < 8; c++) {
            float e[8];
#pragma unroll
            for (int j = 0; j < 8; j++) e[j] = 8 * c + j < OUT ? dy[(8 * c + j) % OUT] : 0.f;
            uint4 q;
            q.x = pack2_sat(e[0], e[1]);
            q.y = pack2_sat(e[2], e[3]);
            q.z = pack2_sat(e[4], e[5]);
            q.w = pack2_sat(e[6], e[7]);
            *reinterpret_cast<uint4 *>(dst + sw128_chunk(t, c)) = q;
          }
        }
        fence_async_smem();
        fence_before();
      }
      if (!(ok = __syncthreads_and(ok))) break;  // every thread leaves together
    }
    if (!ok) break;
    // ---- backward, step l = NH .. 0: the issuer launches dH_l (critical
    // path) and then dW_{l+1}; the rows warps form dZ_{l-1} into tile
    // (l - 1) % 3 once dH_l is done and dW_{l+2}, the last reader of that
    // tile, has completed.  dW_j commits to barW[j & 1]; both of the last
    // two (dW_1, dW_0) commit to barA at step 0.
#pragma unroll 1
    for (int l = NH; l >= 0; l--) {
      if (issuer) {
        fence_after();
        if (l > 0) {  // dH_l = dZ_l W_l: A = dZ_l (K-major over the outputs), B = W_l (MN-major)
          const uint32_t idh = idesc_f16(128, HID, false, true);
          const uint64_t b0 = desc_add(dWmn, T::w_off(l));
          const uint32_t zb = (uint32_t)(l % 3) * 16384;
#pragma unroll 1
          for (int s = 0; s < T::out_(l) / 16; s++)
            mma_f16(tm, desc_add(dZ, zb + 32u * s), desc_add(b0, 2048u * s), idh, s > 0);
          commit(barA);
        }
        // dW_j (+)= dZ_j^T H_j: A = dZ_j (MN-major, 64 outputs), B = H_j (MN-major,
        // blocks of 64 inputs 16384 bytes apart), K = the 128 rows in steps of 16
#pragma unroll 1
        for (int j = l + 1; j >= (l == 0 ? 0 : l + 1); j--) {
          if (j > NH) continue;
          const uint32_t idw = idesc_f16(64, T::in_(j), true, true);
          const uint64_t bh = j == 0 ? dXmn : desc_add(dHmn, (uint32_t)(j - 1) * 16384);
          const uint32_t dcol = tm + (uint32_t)T::dw_col(j), zb = (uint32_t)(j % 3) * 16384;
#pragma unroll 1
          for (int s = 0; s < 8; s++)
            mma_f16(dcol, desc_add(dZmn, zb + 2048u * s), desc_add(bh, 2048u * s), idw, !first || s > 0);
          if (l > 0) commit(barW0 + 8u * (uint32_t)(j & 1));
        }
        if (l == 0) commit(barA);
      }
      if (l > 0 && rows_warp && wait_rows(barA, phA)) {  // dZ_{l-1} = dH_l masked by H_l > 0
        fence_after();
        float v[64];
        tmem_ld64(lane_base, v);
        // dW_{l+2} (committed to barW[l & 1]) last read tile (l - 1) % 3
        if (l + 2 > NH || ((l & 1) ? wait_rows(barW0 + 8, phW1) : wait_rows(barW0, phW0))) {
          const uint8_t *h = sm + T::H_OFF + (uint32_t)(l - 1) * 16384;
          uint8_t *dz = sm + T::DZ_OFF + (uint32_t)((l - 1) % 3) * 16384;
#pragma unroll
          for (int c = 0; c < 8; c++) {
            const uint4 hv = *reinterpret_cast<const uint4 *>(h + sw128_chunk(t, c));
            const uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
            uint32_t q[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const float2 hf = unpack2(hw[j]);
              q[j] = pack2_sat(hf.x > 0.f ? v[8 * c + 2 * j] : 0.f, hf.y > 0.f ? v[8 * c + 2 * j + 1] : 0.f);
            }
            *reinterpret_cast<uint4 *>(dz + sw128_chunk(t, c)) = make_uint4(q[0], q[1], q[2], q[3]);
          }
          fence_async_smem();
          fence_before();
        }
      }
      // step 0: dW_2's phase of barW[0] (if any) is consumed here
      if (l == 0 && NH >= 2 && rows_warp) wait_rows(barW0, phW0);
      if (!(ok = __syncthreads_and(ok))) break;  // every thread leaves together
    }
    if (!ok) break;
    // dW_1 and dW_0 (barA) read X, H_1 and two dZ tiles: complete before the
    // next tile overwrites them
    if (rows_warp) wait_rows(barA, phA);
    ok = __syncthreads_and(ok);
    first = false;
  }
  // ---- this CTA's weight-gradient sums into the gradient.  Layer l's row o
  // is in lane 32 (o / 16) + o % 16 (M = 64 accumulator layout); the rows
  // warps stage every layer in the gradient's own layout in shared memory
  // (H and dZ are free now), then all warps add it to the gradient with
  // coalesced vector reductions.
  float *stage = reinterpret_cast<float *>(sm + T::H_OFF);
  const bool sums = ok && !first;
  if (sums && rows_warp) {
    fence_after();
    const int o = warp * 16 + lane;
#pragma unroll 1
    for (int l = 0; l <= NH; l++) {
      const int K = T::in_(l), N = T::out_(l);
#pragma unroll 1
      for (int c0 = 0; c0 < K; c0 += 64) {
        float v[64];
        tmem_ld64(lane_base + (uint32_t)(T::dw_col(l) + c0), v);
        if (lane < 16 && o < N) {
          float4 *dst = reinterpret_cast<float4 *>(stage + layer_offset(n, l)) + o * (K / 4);
#pragma unroll
          for (int i = 0; i < 64; i += 4)
            if (c0 + i < K) dst[stage_slot(o, (c0 + i) / 4, K / 4)] = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
      }
    }
  }
  __syncthreads();
  if (sums) {
#pragma unroll 1
    for (int l = 0; l <= NH; l++) {
      const int K4 = T::in_(l) / 4, count4 = T::out_(l) * K4, off = layer_offset(n, l);
      const float4 *src = reinterpret_cast<const float4 *>(stage + off);
      for (int q = t; q < count4; q += TC_THREADS) {
        const int o = q / K4, i4 = q - o * K4;
        red_add_v4(n.grad + off + 4 * q, src[o * K4 + stage_slot(o, i4, K4)]);
      }
    }
  }
  if (!ok && t == 0) atomicExch(err, 1);
  if (loss_sum && rows_warp) {
    for (int k = 16; k > 0; k >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, k);
    if (lane == 0) atomicAdd(loss_sum, lsum);
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tm, T::TMEM_COLS);
}

// ------------------------------------------------- inference (tcgen05) ---
// The forward pass alone, for many 128-row tiles per CTA: warps 0-3 own the
// rows and tensor-memory lanes (thread t: row t of the tile), the first
// thread of warp 4 issues the MMAs (M = 128, f32 accumulator in 64 tensor-
// memory columns), the weights arrive by one bulk copy of the weight image.
// Activations ping-pong between two tiles: X and H_2, H_4 .. in tile A,
// H_1, H_3 .. in tile B; layer l reads one and its epilogue writes H_{l+1}
// into the other, whose last reader (layer l - 1's MMAs) has completed.
// Two CTAs share an SM, so one CTA's MMAs overlap the other's loads and
// epilogues.  Io builds row t of the input tile (load, returning what
// store needs) and takes row t's f32 outputs (store).
template <int IN, int NH, int OUT>
struct InferLayout {
  using T = TrainLayout<IN, NH, OUT>;
  static constexpr uint32_t A_OFF = T::W_BYTES;              // X (KB0 blocks), H_2, H_4 ...
  static constexpr uint32_t B_OFF = A_OFF + T::KB0 * 16384;  // H_1, H_3 ...
  static constexpr uint32_t BAR_OFF = B_OFF + 16384;
  static constexpr uint32_t SMEM = BAR_OFF + 64 + 1024;      // + slack for the 1024-byte alignment
  static constexpr uint32_t TMEM_COLS = 64;
  static_assert(A_OFF % 1024 == 0, "operand tiles start on 1024-byte boundaries");
  static_assert(2 * (SMEM + 1024) <= 228 * 1024, "two CTAs per SM");
};

template <int IN, int NH, int OUT, class Io>
__global__ void __launch_bounds__(TC_THREADS, 2)
    k_mlp_infer_tc(const uint8_t *__restrict__ wimg, int rows, Io io, int *err) {
  using T = TrainLayout<IN, NH, OUT>;
  using I = InferLayout<IN, NH, OUT>;
  using namespace tc05;
  extern __shared__ uint8_t tc_raw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
  uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + I::BAR_OFF + 16);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const bool rows_warp = warp < 4;
  const bool issuer = warp == 4 && lane == 0;
  const uint32_t base = smem_addr(sm);
  const uint32_t barA = base + I::BAR_OFF, barL = barA + 8;  // MMA completions; the weight image
  uint32_t phA = 0;
  bool ok = true;
  if (issuer) {
    bar_init(barA, 1);
    bar_init(barL, 1);
    bar_expect_bytes(barL, T::W_BYTES);
    for (uint32_t o = 0; o < T::W_BYTES; o += 16384)
      bulk_copy(base + o, wimg + o, T::W_BYTES - o < 16384 ? T::W_BYTES - o : 16384, barL);
  }
  if (warp == 0) tmem_alloc(tslot, I::TMEM_COLS);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tm = *tslot;
  const uint32_t lane_base = tm + ((uint32_t)((warp & 3) * 32) << 16);
  bool weights = false;  // the issuer has seen the weight image arrive
  const uint64_t dA = desc(base + I::A_OFF, 16, 1024), dB = desc(base + I::B_OFF, 16, 1024);
  const uint64_t dW = desc(base, 16, 1024);
  const int n_tiles = (rows + 127) / 128;
  for (int tile = blockIdx.x; ok && tile < n_tiles; tile += gridDim.x) {
    const int r0 = tile * 128;
    typename Io::Pre pre{};
    if (rows_warp) {
      pre = io.load(r0 + t, r0 + t < rows, sm + I::A_OFF, t);
      fence_async_smem();
    }
    if (issuer && !weights) weights = ok = bar_wait(barL, 0, TC_WAIT_LIMIT);  // overlapped with the first loads
    if (!(ok = __syncthreads_and(ok))) break;  // every thread leaves together
#pragma unroll 1
    for (int l = 0; l <= NH; l++) {
      if (issuer) {
        fence_after();
        const uint64_t a0 = (l & 1) ? dB : dA;
        const uint64_t b0 = desc_add(dW, T::w_off(l));
        const uint32_t id = idesc_f16(128, T::out_(l), false, false);
        const uint32_t bstride = T::out_(l) * 128;  // between the weight tile's 64-input blocks
#pragma unroll 1
        for (int s = 0; s < T::in_(l) / 16; s++)
          mma_f16(tm, desc_add(a0, (uint32_t)(s >> 2) * 16384 + (uint32_t)(s & 3) * 32),
                  desc_add(b0, (uint32_t)(s >> 2) * bstride + (uint32_t)(s & 3) * 32), id, s > 0);
        commit(barA);
      }
      if (rows_warp) {
        const bool got = __all_sync(0xffffffffu, bar_wait(barA, phA, TC_WAIT_LIMIT));
        phA ^= 1;
        ok = ok && got;
        if (got) {
          fence_after();
          float v[64];
          tmem_ld64(lane_base, v);
          if (l < NH) {  // ReLU, f16: row t of H_{l+1}
            uint8_t *dst = sm + (((l + 1) & 1) ? I::B_OFF : I::A_OFF);
#pragma unroll
            for (int c = 0; c < 8; c++) {
              uint4 q;
              q.x = pack2(fmaxf(v[8 * c], 0.f), fmaxf(v[8 * c + 1], 0.f));
              q.y = pack2(fmaxf(v[8 * c + 2], 0.f), fmaxf(v[8 * c + 3], 0.f));
              q.z = pack2(fmaxf(v[8 * c + 4], 0.f), fmaxf(v[8 * c + 5], 0.f));
              q.w = pack2(fmaxf(v[8 * c + 6], 0.f), fmaxf(v[8 * c + 7], 0.f));
              *reinterpret_cast<uint4 *>(dst + sw128_chunk(t, c)) = q;
            }
            fence_async_smem();
          } else {
            io.store(r0 + t, r0 + t < rows, v, pre);
          }
          fence_before();
        }
      }
      if (!(ok = __syncthreads_and(ok))) break;  // every thread leaves together
    }
  }
  // a CTA that stopped early still lets the weight copy land before it exits
  if (issuer && !weights) bar_wait(barL, 0, TC_WAIT_LIMIT);
  if (!ok && t == 0) atomicExch(err, 1);
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tm, I::TMEM_COLS);
}

// Rows of an f16 input matrix X (rows x IN) in, f32 outputs Y (rows x OUT)
// out: the plain forward pass.
template <int IN, int OUT>
struct MatrixIo {
  const __half *X;
  float *Y;
  using Pre = int;
  __device__ Pre load(int row, bool valid, uint8_t *xtile, int t) const {
#pragma unroll
    for (int k8 = 0; k8 < IN / 8; k8++)
      tc05::cp_async16(xtile + (uint32_t)(k8 / 8) * 16384 + tc05::sw128_chunk(t, k8 % 8),
                       X + (size_t)(valid ? row : 0) * IN + k8 * 8, valid ? 16 : 0);
    tc05::cp_async_wait_all();
    return 0;
  }
  __device__ void store(int row, bool valid, const float *v, Pre) const {
    if (!valid) return;
    float4 *y = reinterpret_cast<float4 *>(Y + (size_t)row * OUT);
#pragma unroll
    for (int o = 0; o < OUT / 4; o++) y[o] = make_float4(v[4 * o], v[4 * o + 1], v[4 * o + 2], v[4 * o + 3]);
  }
};

// The weight image the training kernel copies: every f16 weight at its
// swizzled position (after set_params / load_state; Adam keeps it current).
__global__ void k_pack_wimg(Net n, int count, uint8_t *__restrict__ wimg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    *reinterpret_cast<__half *>(wimg + wimg_offset(n, i)) = n.w16[i];
}

// Adam (Kingma & Ba, ICLR 2015) on the f32 master weights; the gradient is
// divided by the loss scale first and cleared afterwards.
__global__ void k_adam(int count, float *__restrict__ w32, __half *__restrict__ w16, float *__restrict__ grad,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2, float eps,
                       float inv_scale, float bc1, float bc2, Net n, uint8_t *__restrict__ wimg) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    if (i == blockIdx.x * blockDim.x + threadIdx.x) {  // first iteration: chained launches (cache training)
      tc05::griddep_launch();
      tc05::griddep_wait();
    }
    float gr = grad[i] * inv_scale;
    if (!isfinite(gr)) gr = 0.f;  // an overflowed element skips this step
    const float mi = b1 * m[i] + (1.f - b1) * gr;
    const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    const float wi = w32[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w32[i] = wi;
    const __half h = __float2half_rn(wi);
    w16[i] = h;
    *reinterpret_cast<__half *>(wimg + wimg_offset(n, i)) = h;  // the training kernel's weight image
    grad[i] = 0.f;
  }
}

// ------------------------------------------------------- path guiding ---
// Network input: one-blob encoding of the position normalised to the scene
// box (3 axes x 32 bins, triangle kernel of one bin width; Mueller et al.,
// "Neural Importance Sampling", ACM TOG 2019) and the surface normal; 99
// values padded to 112.  Output: 8 lobes x (weight logit, kappa
// pre-activation, mean direction xyz), 40 values padded to 48.
constexpr int GUIDE_IN = 112, GUIDE_NH = 3, GUIDE_OUT = 48, GUIDE_LOBES = 8, BLOB_BINS = 32;

// A row of N halves built in registers (fully unrolled encoders), written
// to a 16-byte-aligned row with 16-byte stores.
template <int N>
__device__ __forceinline__ void store_row(const __half (&buf)[N], __half *dst) {
  static_assert(N % 8 == 0, "rows are whole 16-byte chunks");
#pragma unroll
  for (int i = 0; i < N / 8; i++) reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(buf)[i];
}

__device__ __forceinline__ void guide_encode(float3 xn, float3 n, __half *out) {
  const float c[3] = {xn.x, xn.y, xn.z};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float u = fminf(fmaxf(c[a], 0.f), 1.f) * BLOB_BINS;
#pragma unroll
    for (int b = 0; b < BLOB_BINS; b++) out[a * BLOB_BINS + b] = __float2half_rn(fmaxf(0.f, 1.f - fabsf(u - (b + 0.5f))));
  }
  out[96] = __float2half_rn(n.x);
  out[97] = __float2half_rn(n.y);
  out[98] = __float2half_rn(n.z);
#pragma unroll
  for (int i = 99; i < GUIDE_IN; i++) out[i] = __float2half_rn(0.f);
}

// Weighted maximum likelihood of the vMF mixture: loss = -w log q(omega);
// gradient as in oracle/mlp_ref.py vmf_nll_grad.
struct LossVmf {
  const float4 *target;  // (omega.xyz, weight)
  float scale;
  const float *wsum;     // if set: weights are normalised by the batch sum
  float clip;            // if > 0: per-row bound on the gradient's L2 norm (before `scale`)
  static constexpr float KAPPA_MAX = 500.f;
  static constexpr bool kEncodes = false;
  using Pre = float4;  // (omega.xyz, the weight normalised by the batch sum)
  __device__ Pre preload(int row) const {
    float4 tg = target[row];
    tg.w = wsum ? tg.w / fmaxf(*wsum, 1e-30f) : tg.w;
    return tg;
  }
  template <int OUT>
  __device__ float grad(int, const float *y, float *dy, Pre tg) const {
    const float3 w = make_float3(tg.x, tg.y, tg.z);
    float logit[GUIDE_LOBES], kap[GUIDE_LOBES], cs[GUIDE_LOBES], f[GUIDE_LOBES], mn[GUIDE_LOBES];
    float3 mu[GUIDE_LOBES];
    float lmax = -1e30f;
    for (int i = 0; i < GUIDE_LOBES; i++) lmax = fmaxf(lmax, y[5 * i]);
    float zsum = 0.f;
    for (int i = 0; i < GUIDE_LOBES; i++) {
      logit[i] = __expf(y[5 * i] - lmax);
      zsum += logit[i];
      const float kp = y[5 * i + 1];
      kap[i] = fminf((kp > 20.f ? kp : log1pf(__expf(kp))) + 1e-2f, KAPPA_MAX);
      const float3 m = make_float3(y[5 * i + 2], y[5 * i + 3], y[5 * i + 4]);
      mn[i] = fmaxf(sqrtf(m.x * m.x + m.y * m.y + m.z * m.z), 1e-12f);
      mu[i] = make_float3(m.x / mn[i], m.y / mn[i], m.z / mn[i]);
      cs[i] = mu[i].x * w.x + mu[i].y * w.y + mu[i].z * w.z;
    }
    float p = 0.f;
    for (int i = 0; i < GUIDE_LOBES; i++) {
      logit[i] /= zsum;  // pi
      const float e2 = __expf(-2.f * kap[i]);
      f[i] = kap[i] / (6.28318530717958647692f * (1.f - e2)) * __expf(kap[i] * (cs[i] - 1.f));
      p += logit[i] * f[i];
    }
    p = fmaxf(p, 1e-30f);
    const float wn = tg.w;
    if (wn == 0.f) {  // no contribution, no gradient (whatever the outputs)
      for (int o = 0; o < OUT; o++) dy[o] = 0.f;
      return 0.f;
    }
    float n2 = 0.f;
    for (int i = 0; i < GUIDE_LOBES; i++) {
      const float r = logit[i] * f[i] / p;
      const float e2 = __expf(-2.f * kap[i]);
      dy[5 * i] = wn * (logit[i] - r);
      const float dlk = 1.f / kap[i] - 2.f * e2 / (1.f - e2) + (cs[i] - 1.f);
      const bool capped = kap[i] >= KAPPA_MAX;
      dy[5 * i + 1] = capped ? 0.f : wn * (-r * dlk / (1.f + __expf(-y[5 * i + 1])));
      const float k = -r * kap[i] / mn[i];
      dy[5 * i + 2] = wn * k * (w.x - cs[i] * mu[i].x);
      dy[5 * i + 3] = wn * k * (w.y - cs[i] * mu[i].y);
      dy[5 * i + 4] = wn * k * (w.z - cs[i] * mu[i].z);
      for (int c = 0; c < 5; c++) n2 += dy[5 * i + c] * dy[5 * i + c];
    }
    // per-row gradient clipping: a sharp lobe on a heavy record (or a mean
    // vector of tiny norm) must not dominate the step or overflow f16
    const float sc = (clip > 0.f && n2 > clip * clip) ? scale * clip * rsqrtf(n2) : scale;
    for (int o = 0; o < 5 * GUIDE_LOBES; o++) dy[o] *= sc;
    for (int o = 5 * GUIDE_LOBES; o < OUT; o++) dy[o] = 0.f;
    return -wn * logf(p);
  }
};

__device__ __forceinline__ bool finite4(float4 v) {
  return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w);
}

// One guide record (3 float4: position and weight, normal, sampled
// direction) -> its encoded row and its loss target (direction, weight).
// An unusable record (non-finite, or a negative weight) becomes a zero-weight
// row at the box corner.
__device__ __forceinline__ float4 guide_record_row(const float4 *rec, float3 lo, float3 inv_ext, __half *dst) {
  float4 xw = rec[0], nn = rec[1], dd = rec[2];
  if (!(finite4(xw) && finite4(nn) && finite4(dd) && xw.w >= 0.f)) {
    xw = make_float4(lo.x, lo.y, lo.z, 0.f);
    nn = dd = make_float4(0.f, 0.f, 1.f, 0.f);
  }
  const float3 xn = make_float3((xw.x - lo.x) * inv_ext.x, (xw.y - lo.y) * inv_ext.y, (xw.z - lo.z) * inv_ext.z);
  __align__(16) __half row[GUIDE_IN];
  guide_encode(xn, make_float3(nn.x, nn.y, nn.z), row);
  store_row(row, dst);
  return make_float4(dd.x, dd.y, dd.z, xw.w);
}

// Training rows: a random record per row (with replacement), encoded.
__global__ void k_guide_encode_records(const float4 *__restrict__ rec, int count, int rows, uint2 key, uint32_t step,
                                       float3 lo, float3 inv_ext, __half *__restrict__ X, float4 *__restrict__ target,
                                       float *wsum) {
  float part = 0.f;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)r * 0x9E3779B1u ^ (step * 0x85EBCA77u) ^ key.x;
    h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
    const int idx = (int)(h % (uint32_t)count);
    const float4 t = guide_record_row(rec + 3 * (size_t)idx, lo, inv_ext, X + (size_t)r * GUIDE_IN);
    target[r] = t;
    part += t.w;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0 && part != 0.f) atomicAdd(wsum, part);
}

// Grid rows: cell centres x 6 axis normals (+x,-x,+y,-y,+z,-z).
__global__ void k_guide_encode_grid(int res, int rows_valid, int rows, __half *__restrict__ X) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
    __half *out = X + (size_t)r * GUIDE_IN;
    if (r >= rows_valid) {
      for (int i = 0; i < GUIDE_IN; i++) out[i] = __float2half_rn(0.f);
      continue;
    }
    const int bin = r % 6, cell = r / 6;
    const int cx = cell % res, cy = (cell / res) % res, cz = cell / (res * res);
    const float3 xn = make_float3((cx + 0.5f) / res, (cy + 0.5f) / res, (cz + 0.5f) / res);
    const float sgn = (bin & 1) ? -1.f : 1.f;
    const float3 n = make_float3(bin / 2 == 0 ? sgn : 0.f, bin / 2 == 1 ? sgn : 0.f, bin / 2 == 2 ? sgn : 0.f);
    __align__(16) __half row[GUIDE_IN];
    guide_encode(xn, n, row);
    store_row(row, out);
  }
}

// Network outputs -> lobe table rows of GUIDE_ENTRY float4 (the layout the
// renderer reads, see guide_pdf / guide_sample).
__device__ __forceinline__ void guide_row(const float lobe[GUIDE_LOBES][5], float4 *dst) {
  float cdf = 0.f;
  float c[GUIDE_LOBES];
  for (int i = 0; i < GUIDE_LOBES; i++) {
    const float *L = lobe[i];  // {pi, kappa, mu.x, mu.y, mu.z}
    const float k = L[1];
    const float norm = k / (6.28318530717958647692f * -expm1f(-2.f * k));
    const float lc = L[0] > 0.f ? logf(L[0] * norm) - k : -1e30f;
    dst[i] = make_float4(k * L[2], k * L[3], k * L[4], lc);
    cdf += L[0];
    c[i] = cdf;
  }
  c[GUIDE_LOBES - 1] = 1.f;
  dst[8] = make_float4(c[0] / cdf, c[1] / cdf, c[2] / cdf, c[3] / cdf);
  dst[9] = make_float4(c[4] / cdf, c[5] / cdf, c[6] / cdf, 1.f);
}

__global__ void k_guide_post(const float *__restrict__ Y, int rows_valid, float4 *__restrict__ lobes) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows_valid; r += gridDim.x * blockDim.x) {
    const float *y = Y + (size_t)r * GUIDE_OUT;
    float lmax = -1e30f;
    for (int i = 0; i < GUIDE_LOBES; i++) lmax = fmaxf(lmax, y[5 * i]);
    float e[GUIDE_LOBES], z = 0.f;
    for (int i = 0; i < GUIDE_LOBES; i++) {
      e[i] = __expf(y[5 * i] - lmax);
      z += e[i];
    }
    float L[GUIDE_LOBES][5];
    bool ok = z > 0.f && isfinite(z);
    for (int i = 0; i < GUIDE_LOBES; i++) {
      const float kp = y[5 * i + 1];
      const float k = fminf((kp > 20.f ? kp : log1pf(__expf(kp))) + 1e-2f, LossVmf::KAPPA_MAX);
      const float mx = y[5 * i + 2], my = y[5 * i + 3], mz = y[5 * i + 4];
      const float mnorm = sqrtf(mx * mx + my * my + mz * mz);
      L[i][0] = e[i] / z;
      L[i][1] = k;
      L[i][2] = mx / mnorm;
      L[i][3] = my / mnorm;
      L[i][4] = mz / mnorm;
      ok = ok && mnorm > 1e-12f && isfinite(L[i][0]) && isfinite(k) && isfinite(L[i][2]) && isfinite(L[i][3]) &&
           isfinite(L[i][4]);
    }
    if (!ok) {  // one broad lobe: sampling and density stay consistent
      for (int i = 0; i < GUIDE_LOBES; i++) {
        L[i][0] = i == 0 ? 1.f : 0.f;
        L[i][1] = 0.01f;
        L[i][2] = L[i][3] = 0.f;
        L[i][4] = 1.f;
      }
    }
    float4 out[GUIDE_ENTRY];
    guide_row(L, out);
    for (int i = 0; i < GUIDE_ENTRY; i++) lobes[(size_t)r * GUIDE_ENTRY + i] = out[i];
  }
}

// ------------------------------------------------- neural radiance cache --
// Records / queries are 5 float4: (x, roughness), (w_out, 0), (n, 0),
// (albedo, 0), then the training target (rgb, 1) or the query's
// (throughput, pixel bits).
constexpr int NRC_IN = 64, NRC_NH = 5, NRC_OUT = 16;

__device__ __forceinline__ __half fin16(float v) {  // non-finite features encode as 0
  return __float2half_rn(isfinite(v) ? fminf(fmaxf(v, -65504.f), 65504.f) : 0.f);
}

// One-blob encoding (Mueller et al., "Neural Importance Sampling", ACM TOG
// 2019) of u in [0,1] over `bins` bins with a triangular kernel one bin wide.
template <int BINS>
__device__ __forceinline__ void one_blob(float u, __half *out) {
  const float x = fminf(fmaxf(u, 0.f), 1.f) * BINS;  // NaN -> 0
#pragma unroll
  for (int b = 0; b < BINS; b++) out[b] = __float2half_rn(fmaxf(0.f, 1.f - fabsf(x - (b + 0.5f))));
}

// Unit direction -> spherical (theta, phi) in [0,1]^2, one-blob 4 + 4.
__device__ __forceinline__ void dir_blob(float3 d, __half *out) {
  const float th = acosf(fminf(fmaxf(d.z, -1.f), 1.f)) * 0.318309886183790671538f;
  float ph = atan2f(d.y, d.x) * 0.159154943091895335769f;
  ph = ph < 0.f ? ph + 1.f : ph;
  one_blob<4>(th, out);
  one_blob<4>(ph, out + 4);
}

// Cache input (Mueller et al., "Real-time Neural Radiance Caching for Path
// Tracing", ACM TOG 2021): position by a triangle-wave frequency encoding,
// 12 octaves per axis (36); outgoing direction and normal as spherical
// one-blobs (8 + 8); roughness one-blob (4); albedo (3); padded to 64.
__device__ __forceinline__ void nrc_encode(const float4 *f, float3 lo, float3 inv_ext, __half *out) {
  const float c[3] = {(f[0].x - lo.x) * inv_ext.x, (f[0].y - lo.y) * inv_ext.y, (f[0].z - lo.z) * inv_ext.z};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float x = isfinite(c[a]) ? fminf(fmaxf(c[a], 0.f), 1.f) : 0.f;
    float s = x;
#pragma unroll
    for (int k = 0; k < 12; k++, s *= 2.f) {
      const float fr = s - floorf(s);
      out[a * 12 + k] = __float2half_rn(fabsf(2.f * fr - 1.f));
    }
  }
  const float3 wo = make_float3(f[1].x, f[1].y, f[1].z), n = make_float3(f[2].x, f[2].y, f[2].z);
  dir_blob(wo, out + 36);
  dir_blob(n, out + 44);
  one_blob<4>(f[0].w, out + 52);
  out[56] = fin16(f[3].x);
  out[57] = fin16(f[3].y);
  out[58] = fin16(f[3].z);
#pragma unroll
  for (int i = 59; i < NRC_IN; i++) out[i] = __float2half_rn(0.f);
}

// Relative L2 (Mueller et al., "Real-time Neural Radiance Caching for Path
// Tracing", ACM TOG 2021): (y - t)^2 / (sg(y)^2 + 0.01) per channel.
struct LossRelL2 {
  const float4 *target;
  float scale;
  static constexpr bool kEncodes = false;
  using Pre = float4;
  __device__ Pre preload(int row) const { return target[row]; }
  template <int OUT>
  __device__ float grad(int, const float *y, float *dy, Pre t) const {
    const float tv[3] = {t.x, t.y, t.z};
    float loss = 0.f;
    for (int c = 0; c < 3; c++) {
      const float d = y[c] - tv[c];
      const float den = y[c] * y[c] + 0.01f;
      loss += d * d / den;
      dy[c] = scale * 2.f * d / den;
    }
    for (int o = 3; o < OUT; o++) dy[o] = 0.f;
    return loss;
  }
};

// The record a training row draws (with replacement): a hash of the row,
// the Adam step and the render's key.
__device__ __forceinline__ int nrc_record_index(int row, int count, uint32_t key, uint32_t step) {
  uint32_t h = (uint32_t)row * 0x9E3779B1u ^ (step * 0x85EBCA77u) ^ key;
  h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
  return (int)(h % (uint32_t)count);
}

// The cache's training loss with its input built inside the training kernel:
// row r of the batch is record nrc_record_index(r, ...), encoded by
// nrc_encode straight into row t of the swizzled input tile; the target is
// the record's radiance (non-finite: 0).
struct LossRelL2Records {
  const float4 *rec;
  int count;
  uint32_t key, step;
  float3 lo, inv_ext;
  float scale;
  static constexpr bool kEncodes = true;
  using Pre = float4;
  __device__ Pre encode(int row, bool valid, uint8_t *xtile, int t) const {
    __align__(16) __half x[NRC_IN];
    float4 tg = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      const int idx = nrc_record_index(row, count, key, step);
      nrc_encode(rec + 5 * (size_t)idx, lo, inv_ext, x);
      const float4 tt = rec[5 * (size_t)idx + 4];
      if (finite4(tt)) tg = tt;
    } else {
#pragma unroll
      for (int i = 0; i < NRC_IN; i++) x[i] = __float2half_rn(0.f);
    }
#pragma unroll
    for (int c = 0; c < NRC_IN / 8; c++)
      *reinterpret_cast<uint4 *>(xtile + tc05::sw128_chunk(t, c)) = reinterpret_cast<const uint4 *>(x)[c];
    return tg;
  }
  template <int OUT>
  __device__ float grad(int row, const float *y, float *dy, Pre t) const {
    return LossRelL2{nullptr, scale}.template grad<OUT>(row, y, dy, t);
  }
};

// Record r -> row r, without sampling (the encoders as the C ABI exposes
// them).  stride: float4 per record (guide 3; cache records 5, queries 6).
__global__ void k_guide_encode_rows(const float4 *__restrict__ rec, int count, float3 lo, float3 inv_ext,
                                    __half *__restrict__ X, float4 *__restrict__ target) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < count; r += gridDim.x * blockDim.x) {
    const float4 t = guide_record_row(rec + 3 * (size_t)r, lo, inv_ext, X + (size_t)r * GUIDE_IN);
    if (target) target[r] = t;
  }
}

__global__ void k_nrc_encode_rows(const float4 *__restrict__ rec, int count, int stride, float3 lo, float3 inv_ext,
                                  __half *__restrict__ X) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < count; r += gridDim.x * blockDim.x) {
    __align__(16) __half row[NRC_IN];
    nrc_encode(rec + (size_t)stride * r, lo, inv_ext, row);
    store_row(row, X + (size_t)r * NRC_IN);
  }
}

// The cache's queries in (6 float4 each: the vertex features nrc_encode
// reads, then throughput and pixel), throughput x max(cache, 0) out, added
// to the pixel's f32 sum (NaN components as 0, like de_nan).
struct CacheQueryIo {
  const float4 *q;
  float3 lo, inv_ext;
  float4 *accum;
  uint32_t n_pixels;  // accum's length: a query naming a pixel past it is skipped and flagged
  int *bad;
  using Pre = float4;
  __device__ Pre load(int row, bool valid, uint8_t *xtile, int t) const {
    __align__(16) __half x[NRC_IN];
    float4 tq = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) {
      nrc_encode(q + 6 * (size_t)row, lo, inv_ext, x);
      tq = q[6 * (size_t)row + 4];
    } else {
#pragma unroll
      for (int i = 0; i < NRC_IN; i++) x[i] = __float2half_rn(0.f);
    }
#pragma unroll
    for (int c = 0; c < NRC_IN / 8; c++)
      *reinterpret_cast<uint4 *>(xtile + tc05::sw128_chunk(t, c)) = reinterpret_cast<const uint4 *>(x)[c];
    return tq;
  }
  __device__ void store(int, bool valid, const float *v, Pre tq) const {
    if (!valid) return;
    const uint32_t pixel = (uint32_t)__float_as_int(tq.w);
    if (pixel >= n_pixels) {
      atomicExch(bad, 1);
      return;
    }
    float L[3] = {tq.x * fmaxf(v[0], 0.f), tq.y * fmaxf(v[1], 0.f), tq.z * fmaxf(v[2], 0.f)};
#pragma unroll
    for (int c = 0; c < 3; c++) L[c] = isnan(L[c]) ? 0.f : L[c];
    tc05::red_add_v4(reinterpret_cast<float *>(accum + pixel), make_float4(L[0], L[1], L[2], 0.f));
  }
};

}  // namespace mlp
}  // namespace tpt

using namespace tpt;
using namespace tpt::mlp;

// ================================================================ C ABI ===
struct tpt_mlp {
  int device = 0;
  Net net{};
  int in_dim = 0, n_hidden = 0, out_dim = 0;
  int params = 0;
  float *w32 = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  __half *w16 = nullptr;
  uint8_t *wimg = nullptr;   // the f16 weights as the training kernel's swizzled shared-memory image
  int wimg_bytes = 0;
  float *loss = nullptr;
  int *err = nullptr;        // set by the training kernel when an MMA completion wait timed out
  int steps = 0;
};

namespace {

thread_local char g_mlp_err[256] = "";

tpt_status mlp_cuda(cudaError_t e) {
  if (e == cudaSuccess) return TPT_OK;
  std::snprintf(g_mlp_err, sizeof(g_mlp_err), "%s", cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? TPT_ERR_OUT_OF_MEMORY : TPT_ERR_CUDA;
}
#define MLP_CUDA(x)                                  \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) return mlp_cuda(e_);      \
  } while (0)

bool supported(int in, int nh, int out) {
  return (in == 112 && nh == 3 && out == 48) || (in == 64 && nh == 5 && out == 16) || (in == 32 && nh == 2 && out == 16);
}

template <int IN, int NH, int OUT, class Io>
tpt_status launch_infer(tpt_mlp *M, int rows, const Io &io, cudaStream_t s) {
  using L = InferLayout<IN, NH, OUT>;
  if ((int)L::T::W_BYTES != M->wimg_bytes) return TPT_ERR_INVALID_ARGUMENT;
  if (rows <= 0) return TPT_OK;
  int sms = 0;
  MLP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, M->device));
  MLP_CUDA(cudaFuncSetAttribute(k_mlp_infer_tc<IN, NH, OUT, Io>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)L::SMEM));
  const int tiles = (rows + 127) / 128;
  const int grid = tiles < 2 * sms ? tiles : 2 * sms;
  k_mlp_infer_tc<IN, NH, OUT, Io><<<grid, TC_THREADS, L::SMEM, s>>>(M->wimg, rows, io, M->err);
  return mlp_cuda(cudaGetLastError());
}

template <int IN, int NH, int OUT>
tpt_status launch_forward(tpt_mlp *M, const __half *x, int rows, float *y, cudaStream_t s) {
  return launch_infer<IN, NH, OUT>(M, rows, MatrixIo<IN, OUT>{x, y}, s);
}

// A launch that may start while the previous kernel in the stream runs
// (programmatic stream serialisation; the kernel orders itself with
// griddep_wait).
template <typename... K, typename... A>
cudaError_t launch_chained(void (*kern)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// chain_step < 0: a standalone step (its loss sum in M->loss[0], zeroed
// here).  chain_step = k >= 0: step k of a chain of steps each followed by
// adam_step(.., chained): launched to overlap the previous Adam kernel, its
// loss sum in M->loss[k & 1], and it zeroes M->loss[(k + 1) & 1] for the
// next step (the caller zeroes both before step 0).
template <int IN, int NH, int OUT, class Loss>
tpt_status launch_train(tpt_mlp *M, const __half *x, int rows, const Loss &loss, cudaStream_t s, int chain_step = -1) {
  using L = TrainLayout<IN, NH, OUT>;
  static_assert(L::W_BYTES % 16 == 0, "bulk copies move 16-byte multiples");
  if ((int)L::W_BYTES != M->wimg_bytes) return TPT_ERR_INVALID_ARGUMENT;
  int sms = 0;
  MLP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, M->device));
  MLP_CUDA(cudaFuncSetAttribute(k_mlp_train_tc<IN, NH, OUT, Loss>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)L::SMEM));
  const int tiles = (rows + 127) / 128;
  const int grid = tiles < sms ? tiles : sms;
  if (chain_step < 0) {
    MLP_CUDA(cudaMemsetAsync(M->loss, 0, sizeof(float), s));
    k_mlp_train_tc<IN, NH, OUT, Loss><<<grid, TC_THREADS, L::SMEM, s>>>(M->net, M->wimg, x, rows, loss, M->loss,
                                                                        nullptr, M->err);
    return mlp_cuda(cudaGetLastError());
  }
  return mlp_cuda(launch_chained(k_mlp_train_tc<IN, NH, OUT, Loss>, dim3(grid), dim3(TC_THREADS), L::SMEM, s,
                                 M->net, (const uint8_t *)M->wimg, x, rows, loss, M->loss + (chain_step & 1),
                                 M->loss + ((chain_step + 1) & 1), M->err));
}

// Adam on the accumulated gradient (clears it); chained: launched to start
// while the training kernel before it finishes (k_adam waits for it).
tpt_status adam_step(tpt_mlp *M, float lr, float inv_loss_scale, cudaStream_t s, bool chained) {
  M->steps++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float bc1 = 1.f - std::pow(b1, (float)M->steps), bc2 = 1.f - std::pow(b2, (float)M->steps);
  const int grid = (M->params + 255) / 256;
  if (!chained) {
    k_adam<<<grid, 256, 0, s>>>(M->params, M->w32, M->w16, M->grad, M->m, M->v, lr, b1, b2, eps, inv_loss_scale, bc1,
                                bc2, M->net, M->wimg);
    return mlp_cuda(cudaGetLastError());
  }
  return mlp_cuda(launch_chained(k_adam, dim3(grid), dim3(256), 0, s, M->params, M->w32, M->w16, M->grad, M->m, M->v,
                                 lr, b1, b2, eps, inv_loss_scale, bc1, bc2, M->net, M->wimg));
}

// An MMA completion the training kernel waited for in vain: reported once.
tpt_status check_train_err(tpt_mlp *M, cudaStream_t s) {
  int e = 0;
  MLP_CUDA(cudaMemcpyAsync(&e, M->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  if (!e) return TPT_OK;
  MLP_CUDA(cudaMemsetAsync(M->err, 0, sizeof(int), s));
  std::snprintf(g_mlp_err, sizeof(g_mlp_err), "tensor-core MLP kernel: an MMA completion wait timed out");
  return TPT_ERR_CUDA;
}

}  // namespace

namespace tpt {

// Guiding network state used by the guided renderer (kernels.cu).
struct GuideNet {
  tpt_mlp *net = nullptr;
  __half *x = nullptr;
  float *y = nullptr;
  float4 *target = nullptr;
  float *wsum = nullptr;
  int cap_rows = 0;
  float last_loss = 0.f;
};

static tpt_status guide_ws(GuideNet *G, int rows) {
  if (rows <= G->cap_rows) return TPT_OK;
  if (G->x) cudaFree(G->x);
  if (G->y) cudaFree(G->y);
  if (G->target) cudaFree(G->target);
  G->x = nullptr;
  G->y = nullptr;
  G->target = nullptr;
  MLP_CUDA(cudaMalloc(&G->x, (size_t)rows * GUIDE_IN * sizeof(__half)));
  MLP_CUDA(cudaMalloc(&G->y, (size_t)rows * GUIDE_OUT * sizeof(float)));
  MLP_CUDA(cudaMalloc(&G->target, (size_t)rows * sizeof(float4)));
  if (!G->wsum) MLP_CUDA(cudaMalloc(&G->wsum, sizeof(float)));
  G->cap_rows = rows;
  return TPT_OK;
}

tpt_status guide_create(int device, uint64_t seed, GuideNet **out) {
  auto *G = new GuideNet();
  tpt_status st = tpt_mlp_create(device, GUIDE_IN, GUIDE_NH, GUIDE_OUT, seed, &G->net);
  if (st != TPT_OK) {
    delete G;
    return st;
  }
  *out = G;
  return TPT_OK;
}

void guide_destroy(GuideNet *G) {
  if (!G) return;
  tpt_mlp_destroy(G->net);
  if (G->x) cudaFree(G->x);
  if (G->y) cudaFree(G->y);
  if (G->target) cudaFree(G->target);
  if (G->wsum) cudaFree(G->wsum);
  delete G;
}

// `steps` Adam steps on batches of `batch` records drawn from rec[0, count).
tpt_status guide_train(GuideNet *G, const float4 *rec, int count, int steps, int batch, float lr, float3 lo,
                       float3 ext, uint64_t seed, cudaStream_t s) {
  if (count <= 0 || steps <= 0) return TPT_OK;
  batch = (batch + 15) / 16 * 16;
  tpt_status st = guide_ws(G, batch);
  if (st != TPT_OK) return st;
  const float3 inv = make_float3(1.f / ext.x, 1.f / ext.y, 1.f / ext.z);
  const float loss_scale = 256.f;  // weights are normalised to sum 1 per batch
  for (int k = 0; k < steps; k++) {
    MLP_CUDA(cudaMemsetAsync(G->wsum, 0, sizeof(float), s));
    k_guide_encode_records<<<(batch + 255) / 256, 256, 0, s>>>(
        rec, count, batch, make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)), (uint32_t)(G->net->steps + 1), lo,
        inv, G->x, G->target, G->wsum);
    LossVmf L{G->target, loss_scale, G->wsum, 0.25f};
    st = launch_train<GUIDE_IN, GUIDE_NH, GUIDE_OUT>(G->net, G->x, batch, L, s);
    if (st != TPT_OK) return st;
    st = tpt_mlp_adam(G->net, lr, 1.f / loss_scale, s);
    if (st != TPT_OK) return st;
  }
  float l = 0.f;
  MLP_CUDA(cudaMemcpyAsync(&l, G->net->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  G->last_loss = l;  // weighted mean NLL of the last batch
  return check_train_err(G->net, s);
}

// Evaluates the network at every (cell, normal bin) of a res^3 grid and
// writes the lobe table (res^3 * 6 * 8 * 2 float4).
tpt_status guide_refresh(GuideNet *G, int res, float4 *table, cudaStream_t s) {
  const int valid = res * res * res * 6;
  const int rows = (valid + 15) / 16 * 16;
  tpt_status st = guide_ws(G, rows);
  if (st != TPT_OK) return st;
  k_guide_encode_grid<<<(rows + 255) / 256, 256, 0, s>>>(res, valid, rows, G->x);
  st = launch_forward<GUIDE_IN, GUIDE_NH, GUIDE_OUT>(G->net, G->x, rows, G->y, s);
  if (st != TPT_OK) return st;
  k_guide_post<<<(valid + 255) / 256, 256, 0, s>>>(G->y, valid, table);
  return mlp_cuda(cudaGetLastError());
}

float guide_last_loss(const GuideNet *G) { return G->last_loss; }
tpt_mlp *guide_mlp(GuideNet *G) { return G->net; }

// Radiance-cache network state used by the renderer.
// Radiance-cache state: the network only (its training rows are encoded and
// its queries evaluated inside the tensor-core kernels, no workspaces).
struct CacheNet {
  tpt_mlp *net = nullptr;
  float last_loss = 0.f;
};

tpt_status cache_create(int device, uint64_t seed, CacheNet **out) {
  auto *G = new CacheNet();
  tpt_status st = tpt_mlp_create(device, NRC_IN, NRC_NH, NRC_OUT, seed, &G->net);
  if (st != TPT_OK) {
    delete G;
    return st;
  }
  *out = G;
  return TPT_OK;
}

void cache_destroy(CacheNet *G) {
  if (!G) return;
  tpt_mlp_destroy(G->net);
  delete G;
}

tpt_status cache_train(CacheNet *G, const float4 *rec, int count, int steps, int batch, float lr, float3 lo,
                       float3 ext, uint32_t key, cudaStream_t s) {
  if (count <= 0 || steps <= 0) return TPT_OK;
  batch = (batch + 15) / 16 * 16;
  tpt_status st = TPT_OK;
  const float3 inv = make_float3(1.f / ext.x, 1.f / ext.y, 1.f / ext.z);
  const float loss_scale = 1024.f;
  // chained steps: each training kernel's prologue and row encoding overlap
  // the previous step's Adam kernel
  MLP_CUDA(cudaMemsetAsync(G->net->loss, 0, 2 * sizeof(float), s));
  for (int k = 0; k < steps; k++) {
    // the rows are sampled and encoded inside the training kernel
    LossRelL2Records L{rec, count, key, (uint32_t)(G->net->steps + 1), lo, inv, loss_scale / (float)batch};
    st = launch_train<NRC_IN, NRC_NH, NRC_OUT>(G->net, nullptr, batch, L, s, k);
    if (st != TPT_OK) return st;
    if ((st = adam_step(G->net, lr, 1.f / loss_scale, s, true)) != TPT_OK) return st;
  }
  float l = 0.f;
  MLP_CUDA(cudaMemcpyAsync(&l, G->net->loss + ((steps - 1) & 1), sizeof(float), cudaMemcpyDeviceToHost, s));
  MLP_CUDA(cudaStreamSynchronize(s));
  G->last_loss = l / (float)batch;
  return check_train_err(G->net, s);
}

// Evaluates the cache for `count` queries (6 float4 each: the 4 feature
// float4, then (throughput, pixel bits), then unused) and adds throughput x
// max(radiance, 0) to the pixels' sums.
tpt_status cache_infer(CacheNet *G, const float4 *queries, int count, float3 lo, float3 ext, float4 *accum,
                       cudaStream_t s) {
  const float3 inv = make_float3(1.f / ext.x, 1.f / ext.y, 1.f / ext.z);
  // the renderer's own queries name pixels of its frame
  return launch_infer<NRC_IN, NRC_NH, NRC_OUT>(G->net, count,
                                               CacheQueryIo{queries, lo, inv, accum, 0xffffffffu, G->net->err}, s);
}

tpt_status cache_check(CacheNet *G, cudaStream_t s) { return check_train_err(G->net, s); }

float cache_last_loss(const CacheNet *G) { return G->last_loss; }
tpt_mlp *cache_mlp(CacheNet *G) { return G->net; }

int64_t mlp_state_count(const tpt_mlp *M) { return 3 * (int64_t)M->params + 1; }

tpt_status mlp_save_state(const tpt_mlp *M, float *out) {
  const size_t P = (size_t)M->params;
  MLP_CUDA(cudaSetDevice(M->device));
  MLP_CUDA(cudaDeviceSynchronize());  // training runs on the caller's stream
  MLP_CUDA(cudaMemcpy(out, M->w32, P * 4, cudaMemcpyDeviceToHost));
  MLP_CUDA(cudaMemcpy(out + P, M->m, P * 4, cudaMemcpyDeviceToHost));
  MLP_CUDA(cudaMemcpy(out + 2 * P, M->v, P * 4, cudaMemcpyDeviceToHost));
  out[3 * P] = (float)M->steps;
  return TPT_OK;
}

tpt_status mlp_load_state(tpt_mlp *M, const float *in) {
  const size_t P = (size_t)M->params;
  const float steps = in[3 * P];
  if (!(steps >= 0.f && steps < 16777216.f) || steps != (float)(int)steps) return TPT_ERR_INVALID_ARGUMENT;
  tpt_status st = tpt_mlp_set_params(M, in);  // weights (FP32 and FP16), gradient cleared
  if (st != TPT_OK) return st;
  MLP_CUDA(cudaMemcpy(M->m, in + P, P * 4, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(M->v, in + 2 * P, P * 4, cudaMemcpyHostToDevice));
  M->steps = (int)steps;
  return TPT_OK;
}

}  // namespace tpt

extern "C" {

const char *tpt_mlp_last_error(void) { return g_mlp_err; }

tpt_status tpt_mlp_create(int32_t device, int32_t in_dim, int32_t n_hidden, int32_t out_dim, uint64_t seed,
                          tpt_mlp **out) {
  if (!out || !supported(in_dim, n_hidden, out_dim)) return TPT_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return TPT_ERR_NO_DEVICE;
  MLP_CUDA(cudaSetDevice(device));
  auto *M = new tpt_mlp();
  M->device = device;
  M->in_dim = in_dim;
  M->n_hidden = n_hidden;
  M->out_dim = out_dim;
  M->net = Net{in_dim, n_hidden, out_dim, nullptr, nullptr};
  M->params = param_count(M->net);
  const size_t P = (size_t)M->params;
  cudaError_t e = cudaMalloc(&M->w32, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&M->grad, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&M->m, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&M->v, P * 4);
  if (e == cudaSuccess) e = cudaMalloc(&M->w16, P * 2);
  if (e == cudaSuccess) e = cudaMalloc(&M->loss, 2 * sizeof(float));  // two slots for chained steps
  M->wimg_bytes = (int)wimg_bytes(M->net);
  if (e == cudaSuccess) e = cudaMalloc(&M->wimg, (size_t)M->wimg_bytes);
  if (e == cudaSuccess) e = cudaMemset(M->wimg, 0, (size_t)M->wimg_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&M->err, 4);
  if (e == cudaSuccess) e = cudaMemset(M->err, 0, 4);
  if (e != cudaSuccess) {
    tpt_mlp_destroy(M);
    return mlp_cuda(e);
  }
  M->net.w16 = M->w16;
  M->net.grad = M->grad;
  // He-uniform initialisation from a seeded engine
  std::vector<float> w(P);
  std::mt19937_64 rng(seed);
  for (int l = 0; l <= n_hidden; l++) {
    const int K = layer_in(M->net, l), N = layer_out(M->net, l);
    const float lim = std::sqrt(6.0f / (float)K);
    std::uniform_real_distribution<float> U(-lim, lim);
    float *p = w.data() + layer_offset(M->net, l);
    for (int i = 0; i < N * K; i++) p[i] = U(rng);
  }
  *out = M;
  tpt_status st = tpt_mlp_set_params(M, w.data());
  if (st != TPT_OK) {
    tpt_mlp_destroy(M);
    *out = nullptr;
  }
  return st;
}

void tpt_mlp_destroy(tpt_mlp *M) {
  if (!M) return;
  cudaSetDevice(M->device);
  void *ptrs[] = {M->w32, M->grad, M->m, M->v, M->w16, M->wimg, M->loss, M->err};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete M;
}

int64_t tpt_mlp_param_count(const tpt_mlp *M) { return M ? M->params : -1; }

tpt_status tpt_mlp_set_params(tpt_mlp *M, const float *host) {
  if (!M || !host) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  const size_t P = (size_t)M->params;
  std::vector<__half> h(P);
  for (size_t i = 0; i < P; i++) h[i] = __float2half_rn(host[i]);
  MLP_CUDA(cudaMemcpy(M->w32, host, P * 4, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemcpy(M->w16, h.data(), P * 2, cudaMemcpyHostToDevice));
  k_pack_wimg<<<(M->params + 255) / 256, 256>>>(M->net, M->params, M->wimg);
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaMemset(M->grad, 0, P * 4));
  MLP_CUDA(cudaMemset(M->m, 0, P * 4));
  MLP_CUDA(cudaMemset(M->v, 0, P * 4));
  M->steps = 0;
  return TPT_OK;
}

tpt_status tpt_mlp_get_params(const tpt_mlp *M, float *host) {
  if (!M || !host) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  MLP_CUDA(cudaMemcpy(host, M->w32, (size_t)M->params * 4, cudaMemcpyDeviceToHost));
  return TPT_OK;
}

tpt_status tpt_mlp_get_grad(const tpt_mlp *M, float *host) {
  if (!M || !host) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  MLP_CUDA(cudaMemcpy(host, M->grad, (size_t)M->params * 4, cudaMemcpyDeviceToHost));
  return check_train_err(const_cast<tpt_mlp *>(M), nullptr);
}

tpt_status tpt_mlp_forward(tpt_mlp *M, const void *x_f16, int64_t rows, float *y, void *stream) {
  if (!M || !x_f16 || !y || rows <= 0 || rows % 16 || rows > (1 << 28)) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = (cudaStream_t)stream;
  const __half *x = (const __half *)x_f16;
  if (M->in_dim == 112) return launch_forward<112, 3, 48>(M, x, (int)rows, y, s);
  if (M->in_dim == 64) return launch_forward<64, 5, 16>(M, x, (int)rows, y, s);
  return launch_forward<32, 2, 16>(M, x, (int)rows, y, s);
}

tpt_status tpt_mlp_cache_accumulate(tpt_mlp *M, const float *queries, int64_t count, const float *lo,
                                    const float *extent, float *accum, int64_t n_pixels, void *stream) {
  if (!M || !queries || !lo || !extent || !accum || count <= 0 || count > (1 << 28) || n_pixels <= 0 ||
      n_pixels > 0xffffffffll || M->in_dim != NRC_IN || M->n_hidden != NRC_NH || M->out_dim != NRC_OUT)
    return TPT_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; a++)
    if (!(extent[a] > 0.f) || !std::isfinite(lo[a]) || !std::isfinite(extent[a])) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = (cudaStream_t)stream;
  const float3 l = make_float3(lo[0], lo[1], lo[2]);
  const float3 inv = make_float3(1.f / extent[0], 1.f / extent[1], 1.f / extent[2]);
  int *bad = nullptr;  // a query naming a pixel past accum
  MLP_CUDA(cudaMallocAsync((void **)&bad, sizeof(int), s));
  tpt_status st = mlp_cuda(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (st == TPT_OK)
    st = launch_infer<NRC_IN, NRC_NH, NRC_OUT>(
        M, (int)count, CacheQueryIo{(const float4 *)queries, l, inv, (float4 *)accum, (uint32_t)n_pixels, bad}, s);
  int b = 0;
  if (st == TPT_OK) st = mlp_cuda(cudaMemcpyAsync(&b, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(bad, s);
  if (st == TPT_OK) st = check_train_err(M, s);  // synchronises the stream
  if (st == TPT_OK && b) {
    std::snprintf(g_mlp_err, sizeof(g_mlp_err), "cache queries name pixels past n_pixels (skipped)");
    st = TPT_ERR_INVALID_ARGUMENT;
  }
  return st;
}

tpt_status tpt_mlp_backward_given(tpt_mlp *M, const void *x_f16, const float *dy, int64_t rows, float scale,
                                  void *stream) {
  if (!M || !x_f16 || !dy || rows <= 0 || rows % 16 || rows > (1 << 26)) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = (cudaStream_t)stream;
  const __half *x = (const __half *)x_f16;
  LossGiven L{dy, scale};
  if (M->in_dim == 112) return launch_train<112, 3, 48>(M, x, (int)rows, L, s);
  if (M->in_dim == 64) return launch_train<64, 5, 16>(M, x, (int)rows, L, s);
  return launch_train<32, 2, 16>(M, x, (int)rows, L, s);
}

tpt_status tpt_mlp_backward_vmf(tpt_mlp *M, const void *x_f16, const float *target, int64_t rows, float scale,
                                float *loss_out, void *stream) {
  if (!M || !x_f16 || !target || rows <= 0 || rows % 16 || rows > (1 << 26)) return TPT_ERR_INVALID_ARGUMENT;
  if (M->in_dim != GUIDE_IN || M->n_hidden != GUIDE_NH || M->out_dim != GUIDE_OUT) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  tpt_status st = TPT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  LossVmf L{(const float4 *)target, scale, nullptr, 0.f};
  st = launch_train<GUIDE_IN, GUIDE_NH, GUIDE_OUT>(M, (const __half *)x_f16, (int)rows, L, s);
  if (st != TPT_OK) return st;
  if (loss_out) {
    MLP_CUDA(cudaMemcpyAsync(loss_out, M->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    MLP_CUDA(cudaStreamSynchronize(s));
    return check_train_err(M, s);
  }
  return TPT_OK;
}

tpt_status tpt_mlp_backward_rel_l2(tpt_mlp *M, const void *x_f16, const float *target, int64_t rows, float scale,
                                   float *loss_out, void *stream) {
  if (!M || !x_f16 || !target || rows <= 0 || rows % 16 || rows > (1 << 26)) return TPT_ERR_INVALID_ARGUMENT;
  if (M->in_dim != NRC_IN || M->n_hidden != NRC_NH || M->out_dim != NRC_OUT) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  tpt_status st = TPT_OK;
  cudaStream_t s = (cudaStream_t)stream;
  LossRelL2 L{(const float4 *)target, scale};
  st = launch_train<NRC_IN, NRC_NH, NRC_OUT>(M, (const __half *)x_f16, (int)rows, L, s);
  if (st != TPT_OK) return st;
  if (loss_out) {
    MLP_CUDA(cudaMemcpyAsync(loss_out, M->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    MLP_CUDA(cudaStreamSynchronize(s));
    return check_train_err(M, s);
  }
  return TPT_OK;
}

tpt_status tpt_mlp_backward_rel_l2_records(tpt_mlp *M, const float *records, int64_t count, uint32_t key,
                                           uint32_t step, const float *lo, const float *extent, int64_t rows,
                                           float scale, float *loss_out, void *stream) {
  if (!M || !records || !lo || !extent || count <= 0 || count > (1 << 28) || rows <= 0 || rows % 16 ||
      rows > (1 << 26))
    return TPT_ERR_INVALID_ARGUMENT;
  if (M->in_dim != NRC_IN || M->n_hidden != NRC_NH || M->out_dim != NRC_OUT) return TPT_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; a++)
    if (!(extent[a] > 0.f) || !std::isfinite(lo[a]) || !std::isfinite(extent[a])) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  cudaStream_t s = (cudaStream_t)stream;
  const float3 l = make_float3(lo[0], lo[1], lo[2]);
  const float3 inv = make_float3(1.f / extent[0], 1.f / extent[1], 1.f / extent[2]);
  LossRelL2Records L{(const float4 *)records, (int)count, key, step, l, inv, scale};
  tpt_status st = launch_train<NRC_IN, NRC_NH, NRC_OUT>(M, nullptr, (int)rows, L, s);
  if (st != TPT_OK) return st;
  if (loss_out) {
    MLP_CUDA(cudaMemcpyAsync(loss_out, M->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    MLP_CUDA(cudaStreamSynchronize(s));
    return check_train_err(M, s);
  }
  return TPT_OK;
}

static bool encode_args(const float *rec, int64_t count, const float *lo, const float *ext, const void *x) {
  if (!rec || !lo || !ext || !x || count <= 0 || count > (1 << 28)) return false;
  for (int a = 0; a < 3; a++)
    if (!(ext[a] > 0.f) || !std::isfinite(lo[a]) || !std::isfinite(ext[a])) return false;
  return true;
}

tpt_status tpt_guide_encode(const float *records, int64_t count, const float *lo, const float *extent, void *x_f16,
                            float *target, void *stream) {
  if (!encode_args(records, count, lo, extent, x_f16)) return TPT_ERR_INVALID_ARGUMENT;
  const float3 l = make_float3(lo[0], lo[1], lo[2]);
  const float3 inv = make_float3(1.f / extent[0], 1.f / extent[1], 1.f / extent[2]);
  const int grid = (int)std::min<int64_t>((count + 255) / 256, 4096);
  k_guide_encode_rows<<<grid, 256, 0, (cudaStream_t)stream>>>((const float4 *)records, (int)count, l, inv,
                                                              (__half *)x_f16, (float4 *)target);
  return mlp_cuda(cudaGetLastError());
}

tpt_status tpt_nrc_encode(const float *records, int64_t count, int32_t stride, const float *lo, const float *extent,
                          void *x_f16, void *stream) {
  if (!encode_args(records, count, lo, extent, x_f16) || stride < 4) return TPT_ERR_INVALID_ARGUMENT;
  const float3 l = make_float3(lo[0], lo[1], lo[2]);
  const float3 inv = make_float3(1.f / extent[0], 1.f / extent[1], 1.f / extent[2]);
  const int grid = (int)std::min<int64_t>((count + 255) / 256, 4096);
  k_nrc_encode_rows<<<grid, 256, 0, (cudaStream_t)stream>>>((const float4 *)records, (int)count, stride, l, inv,
                                                            (__half *)x_f16);
  return mlp_cuda(cudaGetLastError());
}

tpt_status tpt_mlp_adam(tpt_mlp *M, float lr, float inv_loss_scale, void *stream) {
  if (!M) return TPT_ERR_INVALID_ARGUMENT;
  MLP_CUDA(cudaSetDevice(M->device));
  return adam_step(M, lr, inv_loss_scale, (cudaStream_t)stream, false);
}

}  // extern "C"
