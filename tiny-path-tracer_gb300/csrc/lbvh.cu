// lbvh.cu - GPU linear-BVH build of the opt-in TPT_BVH_LBVH topology.
//
// The reference builds its BVH on the host (bvh_node, hitable.cc:32-56: a
// median split on a random axis).  This builder replaces that topology, for
// scenes compiled with TPT_BVH_LBVH, by a linear BVH built on the device:
//   1. k_lbvh_sort   (one block per job): centroid bounds, 64-bit keys =
//      Morton code of the quantised centroid (Lauterbach et al. 2009) with
//      the primitive index appended (unique keys), bitonic sort in shared
//      memory (global memory for jobs above 16384 primitives);
//   2. k_lbvh_tree   (one thread per internal node): the binary radix tree
//      over the sorted keys (Karras 2012, Algorithm 2): range, split, children
//      and parent links;
//   3. k_lbvh_place  (one thread per internal node): pre-order position = the
//      sum over its ancestors of 1 + (the left subtree's size where the path
//      turns right), and the depth;
//   4. k_lbvh_boxes  (one thread per primitive): boxes bottom-up, the second
//      child to finish computes its parent (an atomic counter per node);
//   5. k_lbvh_finish (one thread per internal node): node_kids (both
//      children's boxes and the pruning size term) and node_skip, and a
//      check that every reference stays inside the job's nodes and the
//      scene's leaves (counted, so a broken tree never reaches a traversal).
// Every step is deterministic (unique keys, min/max unions), so the tree is
// bit-identical to the CPU restatement in the oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include "lbvh.h"

namespace tpt {
namespace {

enum { SORT_THREADS = 1024, SMEM_KEYS = 16384 };

struct Work {
  uint64_t *keys;
  int4 *range;  // internal node: {first, last, split, 0} (job-local)
  int2 *kid;    // children: >= 0 internal node, < 0 ~sorted position
  int *parent_int, *parent_leaf, *pos, *flags, *depth;
};

// The work area in the order lbvh_work_bytes() counts it.
Work carve(void *w, int64_t n_prims, int32_t n_jobs, int64_t n_keys) {
  uint8_t *p = (uint8_t *)w;
  Work k;
  k.keys = (uint64_t *)p;
  p += lbvh_align((size_t)n_keys * 8);
  k.range = (int4 *)p;
  p += lbvh_align((size_t)n_prims * 16);
  k.kid = (int2 *)p;
  p += lbvh_align((size_t)n_prims * 8);
  int **ints[5] = {&k.parent_int, &k.parent_leaf, &k.pos, &k.flags, &k.depth};
  for (int i = 0; i < 5; i++) {
    *ints[i] = (int *)p;
    p += lbvh_align((size_t)(i == 4 ? n_jobs + 1 : n_prims) * 4);
  }
  return k;
}

__device__ __forceinline__ int index_bits(int n) {
  int b = 1;
  while ((1ll << b) < n) b++;
  return b;
}

// the low 21 bits of x moved to every third bit (bit b -> bit 3b)
__device__ __forceinline__ uint64_t spread3(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__device__ __forceinline__ float4 ld4(const f4 *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ float warp_min(float v) {
  for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Sorts keys[0, pad) ascending (bitonic network; pad a power of two).
__device__ void bitonic(uint64_t *K, int pad) {
  for (int k = 2; k <= pad; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < (pad >> 1); t += blockDim.x) {
        const int i = 2 * t - (t & (j - 1));
        const int l = i + j;
        const uint64_t a = K[i], b = K[l];
        if ((a > b) == ((i & k) == 0)) {
          K[i] = b;
          K[l] = a;
        }
      }
      __syncthreads();
    }
}

__global__ void __launch_bounds__(SORT_THREADS) k_lbvh_sort(const i4 *jobs, const f4 *prims, uint64_t *keys) {
  extern __shared__ uint64_t sk[];
  __shared__ float red[6][SORT_THREADS / 32];
  const i4 jb = jobs[blockIdx.x];
  const int n = jb.y, p0 = jb.z;
  uint64_t *gk = keys + jb.w;
  // centroid bounds
  float mn[3], mx[3];
  for (int a = 0; a < 3; a++) {
    mn[a] = __int_as_float(0x7f800000);
    mx[a] = -mn[a];
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float4 lo = ld4(prims + 2 * (p0 + i)), hi = ld4(prims + 2 * (p0 + i) + 1);
    const float c[3] = {__fmul_rn(__fadd_rn(lo.x, hi.x), 0.5f), __fmul_rn(__fadd_rn(lo.y, hi.y), 0.5f),
                        __fmul_rn(__fadd_rn(lo.z, hi.z), 0.5f)};
    for (int a = 0; a < 3; a++) {
      mn[a] = fminf(mn[a], c[a]);
      mx[a] = fmaxf(mx[a], c[a]);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int a = 0; a < 3; a++) {
    mn[a] = warp_min(mn[a]);
    mx[a] = warp_max(mx[a]);
    if (lane == 0) {
      red[a][wid] = mn[a];
      red[3 + a][wid] = mx[a];
    }
  }
  __syncthreads();
  for (int a = 0; a < 3; a++) {
    float lo = red[a][0], hi = red[3 + a][0];
    for (int w = 1; w < nw; w++) {
      lo = fminf(lo, red[a][w]);
      hi = fmaxf(hi, red[3 + a][w]);
    }
    mn[a] = lo;
    mx[a] = hi;
  }
  // keys: Morton code of the centroid in the centroid bounds, then the index
  const int ib = index_bits(n);
  const int mb = min(21, (64 - ib) / 3);
  const float cells = (float)(1u << mb);
  float scale[3];
  for (int a = 0; a < 3; a++) {
    const float ext = __fsub_rn(mx[a], mn[a]);
    scale[a] = ext > 0.f ? __fdiv_rn(cells, ext) : -1.f;
  }
  const int pad = (int)lbvh_pad(n);
  uint64_t *K = pad <= SMEM_KEYS ? sk : gk;
  for (int i = threadIdx.x; i < pad; i += blockDim.x) {
    uint64_t key = ~0ull;
    if (i < n) {
      const float4 lo = ld4(prims + 2 * (p0 + i)), hi = ld4(prims + 2 * (p0 + i) + 1);
      const float c[3] = {__fmul_rn(__fadd_rn(lo.x, hi.x), 0.5f), __fmul_rn(__fadd_rn(lo.y, hi.y), 0.5f),
                          __fmul_rn(__fadd_rn(lo.z, hi.z), 0.5f)};
      uint64_t m = 0;
      for (int a = 0; a < 3; a++) {
        uint32_t q = 0;
        if (scale[a] > 0.f) {
          const float t = __fmul_rn(__fsub_rn(c[a], mn[a]), scale[a]);
          q = t >= cells ? (1u << mb) - 1 : (t >= 0.f ? __float2uint_rz(t) : 0u);
        }
        m |= spread3(q) << (2 - a);
      }
      key = (m << ib) | (uint64_t)i;
    }
    K[i] = key;
  }
  __syncthreads();
  bitonic(K, pad);
  if (K == sk)
    for (int i = threadIdx.x; i < n; i += blockDim.x) gk[i] = sk[i];
}

__device__ __forceinline__ int delta(const uint64_t *K, int n, int i, int j) {
  return j < 0 || j >= n ? -1 : __clzll(K[i] ^ K[j]);
}

__global__ void k_lbvh_tree(const i4 *jobs, const f4 *prims, int n_prims, Work w) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_prims) return;
  const int j = __float_as_int(prims[2 * g + 1].w);
  const i4 jb = jobs[j];
  const int n = jb.y, p0 = jb.z, i = g - p0;
  if (i == 0) w.parent_int[p0] = -1;
  if (n < 2 || i >= n - 1) return;
  const uint64_t *K = w.keys + jb.w;
  const int d = delta(K, n, i, i + 1) - delta(K, n, i, i - 1) > 0 ? 1 : -1;
  const int dmin = delta(K, n, i, i - d);
  int lmax = 2;
  while (delta(K, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(K, n, i, i + (l + t) * d) > dmin) l += t;
  const int jj = i + l * d;
  const int dnode = delta(K, n, i, jj);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (delta(K, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int split = i + s * d + min(d, 0);
  const int first = min(i, jj), last = max(i, jj);
  w.range[g] = make_int4(first, last, split, 0);
  const int left = first == split ? ~split : split;
  const int right = last == split + 1 ? ~(split + 1) : split + 1;
  w.kid[g] = make_int2(left, right);
  if (left >= 0)
    w.parent_int[p0 + left] = i;
  else
    w.parent_leaf[p0 + ~left] = i;
  if (right >= 0)
    w.parent_int[p0 + right] = i;
  else
    w.parent_leaf[p0 + ~right] = i;
}

__global__ void k_lbvh_place(const i4 *jobs, const f4 *prims, int n_prims, Work w) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_prims) return;
  const int j = __float_as_int(prims[2 * g + 1].w);
  const i4 jb = jobs[j];
  const int n = jb.y, p0 = jb.z, i = g - p0;
  if (n < 2 || i >= n - 1) {
    if (n == 1 && i == 0) atomicMax(w.depth + j, 1);
    return;
  }
  int pos = 0, dep = 1, c = i, fc = w.range[g].x;
  for (int guard = 0; guard < n; guard++) {
    const int p = w.parent_int[p0 + c];
    if (p < 0 || p >= n - 1) break;  // the root (links are in range by construction)
    const int4 rp = w.range[p0 + p];
    pos += 1 + (fc == rp.z + 1 ? rp.z - rp.x : 0);  // right child: skip the left subtree
    dep++;
    c = p;
    fc = rp.x;
  }
  w.pos[g] = pos;
  atomicMax(w.depth + j, dep);
}

// Box and reference of child `code` of an internal node.
__device__ __forceinline__ void child_box(const f4 *prims, const f4 *node_lo, const f4 *node_hi, const Work &w,
                                          const uint64_t *K, uint64_t imask, int p0, int base, int code,
                                          float4 &lo, float4 &hi, int &ref) {
  if (code < 0) {
    const int pi = (int)(K[~code] & imask);
    lo = ld4(prims + 2 * (p0 + pi));
    hi = ld4(prims + 2 * (p0 + pi) + 1);
    ref = __float_as_int(lo.w);
  } else {
    ref = base + w.pos[p0 + code];
    lo = __ldcg(reinterpret_cast<const float4 *>(node_lo + ref));
    hi = __ldcg(reinterpret_cast<const float4 *>(node_hi + ref));
  }
}

__global__ void k_lbvh_boxes(const i4 *jobs, const f4 *prims, int n_prims, f4 *node_lo, f4 *node_hi, Work w) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_prims) return;
  const int j = __float_as_int(prims[2 * g + 1].w);
  const i4 jb = jobs[j];
  const int base = jb.x, n = jb.y, p0 = jb.z;
  const uint64_t *K = w.keys + jb.w;
  const uint64_t imask = (1ull << index_bits(n)) - 1;
  if (n == 1) {  // bvh_node with one item: left == right (hitable.cc:37-38)
    float4 lo = ld4(prims + 2 * p0), hi = ld4(prims + 2 * p0 + 1);
    const float ref = lo.w;
    hi.w = ref;
    *reinterpret_cast<float4 *>(node_lo + base) = lo;
    *reinterpret_cast<float4 *>(node_hi + base) = hi;
    return;
  }
  int p = w.parent_leaf[g];
  for (int guard = 0; guard < n && p >= 0 && p < n - 1; guard++) {
    __threadfence();
    if (atomicAdd(w.flags + p0 + p, 1) == 0) return;  // the sibling finishes this node
    __threadfence();
    const int2 kd = w.kid[p0 + p];
    float4 l0, h0, l1, h1;
    int r0, r1;
    child_box(prims, node_lo, node_hi, w, K, imask, p0, base, kd.x, l0, h0, r0);
    child_box(prims, node_lo, node_hi, w, K, imask, p0, base, kd.y, l1, h1, r1);
    const int me = base + w.pos[p0 + p];
    const float4 lo = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), __int_as_float(r0));
    const float4 hi = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), __int_as_float(r1));
    __stcg(reinterpret_cast<float4 *>(node_lo + me), lo);
    __stcg(reinterpret_cast<float4 *>(node_hi + me), hi);
    p = w.parent_int[p0 + p];
  }
}

// node_kids entry of a leaf child: a sphere leaf carries {center, radius}
// and the flag hi.y = 1 (the scene compiler's encoding); other leaves zeros.
__device__ __forceinline__ void leaf_kid(const i4 *leaf_hdr, const f4 *leaf_data, int ref, float4 &lo, float4 &hi) {
  lo = make_float4(0.f, 0.f, 0.f, __int_as_float(ref));
  hi = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!leaf_hdr) return;
  const i4 h = leaf_hdr[~ref];
  if ((h.x & LEAF_TYPE_MASK) == LT_SPHERE) {
    const float4 sp = ld4(leaf_data + h.y);
    lo = make_float4(sp.x, sp.y, sp.z, __int_as_float(ref));
    hi = make_float4(sp.w, 1.f, 0.f, 0.f);
  }
}

__global__ void k_lbvh_finish(const i4 *jobs, const f4 *prims, int n_prims, const f4 *node_lo, const f4 *node_hi,
                              f4 *node_kids, int32_t *node_skip, int n_leaves, const i4 *leaf_hdr,
                              const f4 *leaf_data, int n_jobs, Work w) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_prims) return;
  const int j = __float_as_int(prims[2 * g + 1].w);
  const i4 jb = jobs[j];
  const int base = jb.x, n = jb.y, p0 = jb.z, i = g - p0;
  if (n == 1) {
    if (i == 0) {
      const int ref = __float_as_int(prims[2 * p0].w);
      node_skip[base] = base + 1;
      if (ref >= 0 || ~ref >= n_leaves) {
        atomicAdd(w.depth + n_jobs, 1);
        return;
      }
      float4 lo, hi;
      leaf_kid(leaf_hdr, leaf_data, ref, lo, hi);
      float4 *kd = reinterpret_cast<float4 *>(node_kids + 4 * (size_t)base);
      kd[0] = kd[2] = lo;
      kd[1] = kd[3] = hi;
    }
    return;
  }
  if (i >= n - 1) return;
  const int pos = w.pos[g];
  const int4 r = w.range[g];
  if (pos < 0 || pos >= n - 1 || pos + (r.y - r.x) > n - 1) {  // never, unless the build is broken
    atomicAdd(w.depth + n_jobs, 1);
    return;
  }
  const int me = base + pos;
  node_skip[me] = me + (r.y - r.x);  // the subtree holds last - first internal nodes
  const float4 own_lo = ld4(node_lo + me), own_hi = ld4(node_hi + me);
  const int2 kd = w.kid[g];
  const int refs[2] = {__float_as_int(own_lo.w), __float_as_int(own_hi.w)};
  const int codes[2] = {kd.x, kd.y};
  float4 *out = reinterpret_cast<float4 *>(node_kids + 4 * (size_t)me);
  bool bad = false;
  for (int c = 0; c < 2; c++) {
    float4 lo = make_float4(0.f, 0.f, 0.f, __int_as_float(refs[c])), hi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (codes[c] >= 0) {
      const int cp = codes[c] < n - 1 ? w.pos[p0 + codes[c]] : -1;
      if (cp <= pos || cp >= n - 1 || refs[c] != base + cp) {
        bad = true;
        continue;
      }
      const float4 l = ld4(node_lo + base + cp), h = ld4(node_hi + base + cp);
      lo = make_float4(l.x, l.y, l.z, __int_as_float(base + cp));
      // the box's size term of the pruning bound, in the traversal's order
      const float ext = __fadd_rn(__fadd_rn(__fsub_rn(h.x, l.x), __fsub_rn(h.y, l.y)), __fsub_rn(h.z, l.z));
      hi = make_float4(h.x, h.y, h.z, ext);
    } else if (refs[c] >= 0 || ~refs[c] >= n_leaves) {
      bad = true;
      continue;
    } else {
      leaf_kid(leaf_hdr, leaf_data, refs[c], lo, hi);
    }
    out[2 * c] = lo;
    out[2 * c + 1] = hi;
  }
  if (bad) atomicAdd(w.depth + n_jobs, 1);
}

}  // namespace

int32_t *lbvh_depths(void *work, int64_t n_prims, int32_t n_jobs, int64_t n_keys) {
  return carve(work, n_prims, n_jobs, n_keys).depth;
}

cudaError_t lbvh_build(const LbvhArgs &a, cudaStream_t s) {
  if (a.n_jobs <= 0 || a.n_prims <= 0) return cudaSuccess;
  const Work w = carve(a.work, a.n_prims, a.n_jobs, a.n_keys);
  cudaError_t e = cudaMemsetAsync(w.flags, 0, (size_t)a.n_prims * 4, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.depth, 0, (size_t)(a.n_jobs + 1) * 4, s);
  if (e != cudaSuccess) return e;
  const int smem = (int)(8 * (int64_t)(a.max_pad < SMEM_KEYS ? a.max_pad : SMEM_KEYS));
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k_lbvh_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  k_lbvh_sort<<<a.n_jobs, SORT_THREADS, smem, s>>>(a.jobs, a.prims, w.keys);
  const int grid = (a.n_prims + 255) / 256;
  k_lbvh_tree<<<grid, 256, 0, s>>>(a.jobs, a.prims, a.n_prims, w);
  k_lbvh_place<<<grid, 256, 0, s>>>(a.jobs, a.prims, a.n_prims, w);
  k_lbvh_boxes<<<grid, 256, 0, s>>>(a.jobs, a.prims, a.n_prims, a.node_lo, a.node_hi, w);
  k_lbvh_finish<<<grid, 256, 0, s>>>(a.jobs, a.prims, a.n_prims, a.node_lo, a.node_hi, a.node_kids, a.node_skip,
                                     a.n_leaves, a.leaf_hdr, a.leaf_data, a.n_jobs, w);
  return cudaGetLastError();
}

}  // namespace tpt
