/*
 * lbvh.cc - CPU restatement of the GPU linear-BVH build (TPT_BVH_LBVH).
 *
 * TEST INFRASTRUCTURE ONLY: the tests compare the product's GPU builder
 * (tiny-path-tracer_gb300/csrc/lbvh.cu) against it.  The reference has no such builder
 * (its bvh_node, hitable.cc:32-56, splits at the median of a random axis on
 * the host); this is the opt-in alternative topology, restated from the
 * published algorithm:
 *   - Morton keys of the primitive box centroids, quantised to the centroid
 *     bounds (Lauterbach et al. 2009, "Fast BVH Construction on GPUs"), with
 *     the primitive's index appended so every key is unique;
 *   - the binary radix tree over the sorted keys (Karras 2012, "Maximizing
 *     Parallelism in the Construction of BVHs, Octrees, and k-d Trees",
 *     Algorithm 2);
 *   - boxes bottom-up, nodes laid out in pre-order.
 * The float arithmetic is written so that the host (-ffp-contract=off) and
 * the device (explicit round-to-nearest intrinsics) produce the same bits.
 */
#include <algorithm>
#include <cstdint>
#include <vector>

#include "oracle.h"

namespace {

// 21, 20, ... bits of x spread to every third bit.
uint64_t spread3(uint64_t x) {
  uint64_t r = 0;
  for (int b = 0; b < 21; b++) r |= ((x >> b) & 1ull) << (3 * b);
  return r;
}

int index_bits(int n) {
  int b = 1;
  while ((1ll << b) < n) b++;
  return b;
}

int clz64(uint64_t x) {
  if (!x) return 64;
  int n = 0;
  while (!(x & (1ull << 63))) {
    x <<= 1;
    n++;
  }
  return n;
}

}  // namespace

extern "C" {

int32_t oracle_lbvh_keys(const float *boxes, int32_t n, uint64_t *keys) {
  if (n < 1) return -1;
  // centroid bounds
  std::vector<float> c(3 * (size_t)n);
  for (int i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) c[3 * i + a] = (boxes[6 * i + a] + boxes[6 * i + 3 + a]) * 0.5f;
  float cmin[3] = {c[0], c[1], c[2]}, cmax[3] = {c[0], c[1], c[2]};
  for (int i = 1; i < n; i++)
    for (int a = 0; a < 3; a++) {
      cmin[a] = std::min(cmin[a], c[3 * i + a]);
      cmax[a] = std::max(cmax[a], c[3 * i + a]);
    }
  const int ib = index_bits(n);
  const int mb = std::min(21, (64 - ib) / 3);
  const float cells = (float)(1u << mb);
  for (int i = 0; i < n; i++) {
    uint64_t m = 0;
    for (int a = 0; a < 3; a++) {
      const float ext = cmax[a] - cmin[a];
      uint32_t q = 0;
      if (ext > 0.f) {
        const float t = (c[3 * i + a] - cmin[a]) * (cells / ext);
        q = t >= cells ? (1u << mb) - 1 : (t >= 0.f ? (uint32_t)t : 0u);
      }
      m |= spread3(q) << (2 - a);  // x in the highest bit of each triple
    }
    keys[i] = (m << ib) | (uint64_t)i;
  }
  return mb;
}

int32_t oracle_lbvh_build(const float *boxes, int32_t n, float *out_boxes, int32_t *out_kids, int32_t *out_skip,
                          int32_t *out_depth) {
  if (n < 1) return -1;
  const int ib = index_bits(n);
  std::vector<uint64_t> keys(n);
  oracle_lbvh_keys(boxes, n, keys.data());
  std::sort(keys.begin(), keys.end());
  const uint64_t imask = (1ull << ib) - 1;
  std::vector<int> prim(n);
  for (int i = 0; i < n; i++) prim[i] = (int)(keys[i] & imask);
  if (n == 1) {
    for (int k = 0; k < 6; k++) out_boxes[k] = boxes[k];
    out_kids[0] = out_kids[1] = ~prim[0];
    out_skip[0] = 1;
    *out_depth = 1;
    return 1;
  }
  auto delta = [&](int i, int j) { return j < 0 || j >= n ? -1 : clz64(keys[i] ^ keys[j]); };
  // Karras 2012: internal node i spans [first, last] and splits after gamma
  const int m = n - 1;
  std::vector<int> first(m), last(m), gamma(m), kid(2 * m);
  for (int i = 0; i < m; i++) {
    const int d = delta(i, i + 1) - delta(i, i - 1) > 0 ? 1 : -1;
    const int dmin = delta(i, i - d);
    int lmax = 2;
    while (delta(i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
      if (delta(i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(i, j);
    int s = 0, t = l;
    do {
      t = (t + 1) >> 1;
      if (delta(i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int g = i + s * d + std::min(d, 0);
    first[i] = std::min(i, j);
    last[i] = std::max(i, j);
    gamma[i] = g;
    kid[2 * i] = first[i] == g ? ~g : g;              // leaf g or internal g
    kid[2 * i + 1] = last[i] == g + 1 ? ~(g + 1) : g + 1;
  }
  // pre-order: node, left subtree (gamma - first internal nodes), right subtree
  std::vector<int> pos(m), depth(m);
  std::vector<float> box(6 * (size_t)m);
  int max_depth = 0;
  struct Frame {
    int node, p, dep;
  };
  std::vector<Frame> st{{0, 0, 1}};
  while (!st.empty()) {
    const Frame f = st.back();
    st.pop_back();
    pos[f.node] = f.p;
    depth[f.node] = f.dep;
    max_depth = std::max(max_depth, f.dep);
    const int i = f.node;
    if (kid[2 * i + 1] >= 0) st.push_back({kid[2 * i + 1], f.p + 1 + (gamma[i] - first[i]), f.dep + 1});
    if (kid[2 * i] >= 0) st.push_back({kid[2 * i], f.p + 1, f.dep + 1});
  }
  // boxes bottom-up (children have larger pre-order positions)
  std::vector<int> by_pos(m);
  for (int i = 0; i < m; i++) by_pos[pos[i]] = i;
  for (int p = m - 1; p >= 0; p--) {
    const int i = by_pos[p];
    float b[2][6];
    for (int c = 0; c < 2; c++) {
      const int k = kid[2 * i + c];
      const float *src = k < 0 ? boxes + 6 * (size_t)prim[~k] : &box[6 * (size_t)k];
      for (int a = 0; a < 6; a++) b[c][a] = src[a];
    }
    for (int a = 0; a < 3; a++) {
      box[6 * (size_t)i + a] = std::min(b[0][a], b[1][a]);
      box[6 * (size_t)i + 3 + a] = std::max(b[0][3 + a], b[1][3 + a]);
    }
  }
  for (int i = 0; i < m; i++) {
    const int p = pos[i];
    for (int a = 0; a < 6; a++) out_boxes[6 * p + a] = box[6 * (size_t)i + a];
    for (int c = 0; c < 2; c++) {
      const int k = kid[2 * i + c];
      out_kids[2 * p + c] = k < 0 ? ~prim[~k] : pos[k];
    }
    out_skip[p] = p + (last[i] - first[i]);
  }
  *out_depth = max_depth;
  return m;
}

}  // extern "C"
