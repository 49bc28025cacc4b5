// kernels.cu - sm_103a kernels of the hot path and the device half of the
// C ABI (context, scene upload, batched closest hit, render).
//
// Render engines (same device functions, different schedulers):
//   wavefront   generate -> [traverse -> shade]* with path regeneration:
//               SoA path state in two ping-pong buffers, paths that survive a
//               bounce or that replace a finished path are compacted into the
//               other buffer with __ballot_sync + one atomic per warp; the
//               iteration pair is replayed from a CUDA graph.
//   persistent  one launch of SM-count x occupancy blocks; each warp claims
//               camera samples from a global counter (one atomic per warp)
//               and carries its paths to termination in registers.
// Both accumulate into a float4 image buffer (optionally also double) with
// vector atomics; `resolve` divides by spp.  No kernel waits on another and
// every loop is bounded by the sample count and max_depth.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/tpt.h"
#include "arena.h"
#include "device.cuh"
#include "learn_internal.h"
#include "scene_internal.h"

namespace tpt {

// ------------------------------------------------------------ counters ----
struct WfCounters {
  unsigned int count[2];        // live paths in each ping-pong buffer
  unsigned long long issued;    // camera samples handed out
  unsigned long long segments;  // rays traced
  int err;
  int pad;
};

// SoA path state (64 bytes per path).
struct PathBuf {
  float4 *o_time;   // origin, ray time
  float4 *d_depth;  // direction, bounce depth (int bits)
  float4 *thr_pix;  // throughput, pixel (int bits)
  float4 *rad_smp;  // radiance so far, sample index (int bits)
  int4 *aux;        // learned renders: training-record slots of the path (else unused)
};

__device__ __forceinline__ void warp_claim(bool want, unsigned long long *counter, unsigned long long &base,
                                           int &rank) {
  const unsigned mask = __ballot_sync(0xffffffffu, want);
  const int lane = threadIdx.x & 31;
  rank = __popc(mask & ((1u << lane) - 1u));
  unsigned long long b = 0;
  const int leader = mask ? __ffs(mask) - 1 : 0;
  if (want && lane == leader) b = atomicAdd(counter, (unsigned long long)__popc(mask));
  base = __shfl_sync(0xffffffffu, b, leader);
}

// Whether the warp's idle lanes take new camera samples now: when at least
// `refill` of them are idle (1: at once, each lane on its own; 32: only when
// the whole warp is idle, so a warp's paths stay at the same depth over
// neighbouring pixels, as in a wavefront), or when no lane is left tracing.
__device__ __forceinline__ bool refill_now(bool want, bool alive, int refill) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  return m && ((int)__popc(m) >= refill || !__any_sync(0xffffffffu, alive));
}

__device__ __forceinline__ unsigned warp_append(bool want, unsigned int *counter) {
  const unsigned mask = __ballot_sync(0xffffffffu, want);
  const int lane = threadIdx.x & 31;
  const int rank = __popc(mask & ((1u << lane) - 1u));
  unsigned b = 0;
  const int leader = mask ? __ffs(mask) - 1 : 0;
  if (want && lane == leader) b = atomicAdd(counter, (unsigned)__popc(mask));
  b = __shfl_sync(0xffffffffu, b, leader);
  return b + rank;
}

struct FrameDesc {
  int nx, ny, spp;
  unsigned long long total;  // nx*ny*spp
  float4 *accum;             // per pixel sum (xyz)
  double *accum64;           // optional per pixel double sum (3 per pixel)
};

// sample index s -> (pixel, sample number): pixel-major within a pass so a
// warp's camera rays are neighbours.
__device__ __forceinline__ void sample_coords(const FrameDesc &F, unsigned long long s, uint32_t &pixel,
                                              uint32_t &sample, int &i, int &j) {
  const unsigned long long npix = (unsigned long long)F.nx * F.ny;
  sample = (uint32_t)(s / npix);
  pixel = (uint32_t)(s - (unsigned long long)sample * npix);
  const int row = (int)(pixel / (uint32_t)F.nx);  // 0 = top row
  i = (int)(pixel - (uint32_t)row * F.nx);
  j = F.ny - 1 - row;
}

__device__ __forceinline__ void accumulate(const FrameDesc &F, uint32_t pixel, float3 L) {
  L = de_nan(L);
  atomicAdd(F.accum + pixel, make_float4(L.x, L.y, L.z, 0.f));
  if (F.accum64) {
    atomicAdd(F.accum64 + 3 * (size_t)pixel, (double)L.x);
    atomicAdd(F.accum64 + 3 * (size_t)pixel + 1, (double)L.y);
    atomicAdd(F.accum64 + 3 * (size_t)pixel + 2, (double)L.z);
  }
}

__device__ __forceinline__ void write_path(const PathBuf &B, unsigned idx, const Ray &r, int depth, float3 T,
                                           float3 L, uint32_t pixel, uint32_t sample) {
  B.o_time[idx] = make_float4(r.o.x, r.o.y, r.o.z, r.time);
  B.d_depth[idx] = make_float4(r.d.x, r.d.y, r.d.z, __int_as_float(depth));
  B.thr_pix[idx] = make_float4(T.x, T.y, T.z, __int_as_float((int)pixel));
  B.rad_smp[idx] = make_float4(L.x, L.y, L.z, __int_as_float((int)sample));
}

// ---------------------------------------------------------------- kernels -

// Batched world->hit for the parity boundary (tpt_trace_closest).
template <int FEAT>
__global__ void k_trace_closest(DevScene S, const float *__restrict__ rays, long long n, uint2 key,
                                float *__restrict__ hit_f, int *__restrict__ hit_i, int *err) {
  extern __shared__ int2 stack_smem[];
  int2 *stk = stack_smem + threadIdx.x;
  int e = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const float *q = rays + 7 * k;
    Ray r{v3(q[0], q[1], q[2]), v3(q[3], q[4], q[5]), q[6]};
    MediumRng m{make_uint4((uint32_t)k, (uint32_t)(k >> 32), 0u, 0x4d454449u), key, 0};
    HitRef h;
    float *o = hit_f + 9 * k;
    if (trace_closest<FEAT>(S, r, 0.001f, stk, blockDim.x, m, h, e)) {
      Surface sf;
      finalize(S, r, h, sf);
      o[0] = h.t; o[1] = sf.u; o[2] = sf.v;
      o[3] = sf.p.x; o[4] = sf.p.y; o[5] = sf.p.z;
      o[6] = sf.n.x; o[7] = sf.n.y; o[8] = sf.n.z;
      hit_i[2 * k] = 1;
      hit_i[2 * k + 1] = S.leaf_user[h.leaf];
    } else {
      for (int c = 0; c < 9; c++) o[c] = 0.f;
      hit_i[2 * k] = 0;
      hit_i[2 * k + 1] = -1;
    }
  }
  if (e) atomicExch(err, e);
}

// Fills slots [0, count) of a path buffer with camera samples first..first+count.
__global__ void k_wf_generate(DevScene S, FrameDesc F, PathBuf out, unsigned long long first, unsigned count,
                              uint2 key) {
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    uint32_t pixel, sample;
    int i, j;
    sample_coords(F, first + k, pixel, sample, i, j);
    const Ray r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, key);
    write_path(out, k, r, 0, v3(1.f, 1.f, 1.f), v3(0.f, 0.f, 0.f), pixel, sample);
  }
}

// Closest hit for every live path of buffer `cur`; also clears the append
// counter of the other buffer for the following shade pass.
template <int FEAT = FEAT_ALL>
__global__ void k_wf_traverse(DevScene S, PathBuf in, int cur, WfCounters *C, int4 *__restrict__ hits, uint2 key) {
  extern __shared__ int2 stack_smem[];
  int2 *stk = stack_smem + threadIdx.x;
  const unsigned n = C->count[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    C->count[cur ^ 1] = 0;
    C->segments += n;
  }
  int e = 0;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float4 ot = in.o_time[k], dd = in.d_depth[k];
    const float4 tp = in.thr_pix[k], rs = in.rad_smp[k];
    const Ray r{v3(ot.x, ot.y, ot.z), v3(dd.x, dd.y, dd.z), ot.w};
    MediumRng m{make_uint4((uint32_t)__float_as_int(tp.w), (uint32_t)__float_as_int(rs.w),
                           (uint32_t)__float_as_int(dd.w), 0u), key, 1};
    HitRef h;
    if (trace_closest<FEAT>(S, r, 0.001f, stk, blockDim.x, m, h, e))
      hits[k] = make_int4(__float_as_int(h.t), h.leaf, h.inst, h.face);
    else
      hits[k] = make_int4(0, -1, -1, -1);
  }
  if (e) atomicExch(&C->err, e);
}

// Shades every live path of buffer `cur`; survivors and regenerated camera
// paths are appended (compacted) to buffer cur^1; finished paths are
// accumulated.
__global__ void k_wf_shade(DevScene S, RenderCfg cfg, FrameDesc F, PathBuf in, PathBuf out, int cur, WfCounters *C,
                           const int4 *__restrict__ hits) {
  const unsigned n = C->count[cur];
  const unsigned stride = gridDim.x * blockDim.x;
  // whole warps iterate together (ballots need converged lanes)
  const unsigned n_round = (n + 31u) & ~31u;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n_round; k += stride) {
    const bool live = k < n;
    bool cont = false;
    Ray r{};
    int depth = 0;
    float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
    uint32_t pixel = 0, sample = 0;
    if (live) {
      const float4 ot = in.o_time[k], dd = in.d_depth[k];
      const float4 tp = in.thr_pix[k], rs = in.rad_smp[k];
      r = Ray{v3(ot.x, ot.y, ot.z), v3(dd.x, dd.y, dd.z), ot.w};
      depth = __float_as_int(dd.w);
      T = v3(tp.x, tp.y, tp.z);
      L = v3(rs.x, rs.y, rs.z);
      pixel = (uint32_t)__float_as_int(tp.w);
      sample = (uint32_t)__float_as_int(rs.w);
      const int4 hv = hits[k];
      const HitRef h{__int_as_float(hv.x), hv.y, hv.z, hv.w};
      cont = shade_vertex(S, cfg, r, hv.y >= 0, h, T, L, depth, pixel, sample);
      if (cont) {
        depth++;
      } else {
        accumulate(F, pixel, L);
      }
    }
    // regenerate finished paths from the global sample counter
    const bool want = live && !cont;
    unsigned long long base;
    int rank;
    warp_claim(want, &C->issued, base, rank);
    bool fresh = false;
    if (want) {
      const unsigned long long s = base + (unsigned long long)rank;
      if (s < F.total) {
        int i, j;
        sample_coords(F, s, pixel, sample, i, j);
        r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, cfg.key);
        depth = 0;
        T = v3(1.f, 1.f, 1.f);
        L = v3(0.f, 0.f, 0.f);
        fresh = true;
      }
    }
    const bool emit = cont || fresh;
    const unsigned slot = warp_append(emit, &C->count[cur ^ 1]);
    if (emit) write_path(out, slot, r, depth, T, L, pixel, sample);
  }
}

// Learned renders on the wavefront engine: the per-pass sample mapping, the
// training-record buffers and the cache queries (one struct for both modes).
struct WfLearn {
  GuideView gv;                       // guided: lobe table (lobes == nullptr: plain mixture)
  unsigned long long sample_offset;   // claimed index s -> sample_coords(F, s + sample_offset)
  uint32_t sample_add;                // added to the sample number (guided passes)
  uint32_t stride;                    // guided: every stride-th sample records; cache: trains
  float4 *records;                    // guided: 3 float4 per record (ring); cache: 5 float4 (capped)
  unsigned *rec_count;
  unsigned rec_cap;
  float4 *pend;                       // guided: 5 float4 per recording path; cache: T_k, L_k per record
  unsigned *pend_count;
  int term_depth;                     // cache
  float spread_sqrt_c;                // cache: sqrt(c) of the path-spread rule (0: off)
  float4 *queries;                    // cache: 6 float4 per query
  unsigned *q_count;
  unsigned q_cap;
};

__device__ __forceinline__ bool wf_training(const FrameDesc &F, const WfLearn &W, uint32_t pixel, uint32_t sample) {
  const unsigned long long npix = (unsigned long long)F.nx * F.ny;
  return ((unsigned long long)(sample - W.sample_add) * npix + pixel) % W.stride == 0;
}
// A path's aux.w: the training flag (decided once, when the path is
// generated: the 64-bit modulo above is too costly per vertex) and, for the
// cache, the count of its records in the low bits.  aux.xyz: a training
// path's record slots; for the cache's other paths, under the path-spread
// rule, the Spread state (thr, sum, pdf as float bits).
enum { AUX_TRAIN = 1 << 8, AUX_COUNT = 0xff };
__device__ __forceinline__ int4 fresh_aux(const FrameDesc &F, const WfLearn &W, uint32_t pixel, uint32_t sample) {
  const bool training = wf_training(F, W, pixel, sample);
  if (!training && W.spread_sqrt_c > 0.f) return make_int4(__float_as_int(W.spread_sqrt_c), 0, 0, 0);
  return make_int4(-1, -1, -1, training ? AUX_TRAIN : 0);
}
// Path guiding needs only the pending-record slot and the training flag: one
// int per path instead of the int4 (bits 0-29: slot + 1, bit 30: training),
// which spares the shade kernel 24 B of the path state's traffic each way.
__device__ __forceinline__ int pack_aux1(const int4 &a) { return (a.x + 1) | ((a.w & AUX_TRAIN) ? (1 << 30) : 0); }
__device__ __forceinline__ int4 unpack_aux1(int v) {
  return make_int4((v & 0x3fffffff) - 1, -1, -1, (v >> 30) & 1 ? AUX_TRAIN : 0);
}
template <int MODE>
__device__ __forceinline__ int4 load_aux(const PathBuf &b, unsigned k) {
  if (MODE == 1) return unpack_aux1(reinterpret_cast<const int *>(b.aux)[k]);
  return b.aux[k];
}
template <int MODE>
__device__ __forceinline__ void store_aux(const PathBuf &b, unsigned k, const int4 &a) {
  if (MODE == 1)
    reinterpret_cast<int *>(b.aux)[k] = pack_aux1(a);
  else
    b.aux[k] = a;
}

// Fills slots [0, count) with camera samples first..first+count of a learned pass.
template <int MODE>
__global__ void k_wf_generate_learn(DevScene S, FrameDesc F, PathBuf out, unsigned count, uint2 key, WfLearn W) {
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    uint32_t pixel, sample;
    int i, j;
    sample_coords(F, k + W.sample_offset, pixel, sample, i, j);
    sample += W.sample_add;
    const Ray r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, key);
    write_path(out, k, r, 0, v3(1.f, 1.f, 1.f), v3(0.f, 0.f, 0.f), pixel, sample);
    store_aux<MODE>(out, k, fresh_aux(F, W, pixel, sample));
  }
}

// k_wf_shade for the learned renders.  MODE 1: path guiding (guided sampling
// at diffuse vertices; a recording path keeps its first diffuse vertex in
// `pend` and emits the finished record when it ends).  MODE 2: radiance
// cache (paths end at the first diffuse vertex past term_depth and leave a
// query; training paths record their first three diffuse vertices and fill
// in the targets when they end).  Same per-vertex arithmetic as the
// persistent engines (shade_vertex_t).
template <int MODE>
__global__ void k_wf_shade_learn(DevScene S, RenderCfg cfg, FrameDesc F, PathBuf in, PathBuf out, int cur,
                                 WfCounters *C, const int4 *__restrict__ hits, WfLearn W) {
  const unsigned n = C->count[cur];
  const unsigned stride = gridDim.x * blockDim.x;
  const unsigned n_round = (n + 31u) & ~31u;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n_round; k += stride) {
    const bool live = k < n;
    bool cont = false;
    Ray r{};
    int depth = 0;
    float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
    uint32_t pixel = 0, sample = 0;
    int4 aux = make_int4(-1, -1, -1, 0);
    bool new_rec = false, want_q = false, want_r = false;
    GuideRec grec{};
    VertexInfo vi{};
    float3 Tb = T, Lb = L;
    if (live) {
      const float4 ot = in.o_time[k], dd = in.d_depth[k];
      const float4 tp = in.thr_pix[k], rs = in.rad_smp[k];
      r = Ray{v3(ot.x, ot.y, ot.z), v3(dd.x, dd.y, dd.z), ot.w};
      depth = __float_as_int(dd.w);
      T = v3(tp.x, tp.y, tp.z);
      L = v3(rs.x, rs.y, rs.z);
      pixel = (uint32_t)__float_as_int(tp.w);
      sample = (uint32_t)__float_as_int(rs.w);
      aux = load_aux<MODE>(in, k);
      Tb = T;
      Lb = L;
      const int4 hv = hits[k];
      const HitRef h{__int_as_float(hv.x), hv.y, hv.z, hv.w};
      const bool training = (aux.w & AUX_TRAIN) != 0;
      if (MODE == 1) {
        grec.valid = aux.x >= 0 || !training;  // only recording paths without a record yet take one
        const bool had = grec.valid;
        cont = shade_vertex_t<true>(S, cfg, r, hv.y >= 0, h, T, L, depth, pixel, sample, W.gv, grec);
        new_rec = !had && grec.valid && finite3(grec.x) && finite3(grec.n) && finite3(grec.d);
      } else {
        const bool spread = !training && W.spread_sqrt_c > 0.f;
        const bool may_query = !training && (depth >= W.term_depth || spread);
        const bool rec_here = training && hv.y >= 0 && (aux.w & AUX_COUNT) < 3;
        bool queried = false;
        Spread sp{__int_as_float(aux.x), __int_as_float(aux.y), __int_as_float(aux.z)};
        cont = shade_vertex_t<false>(S, cfg, r, hv.y >= 0, h, T, L, depth, pixel, sample, W.gv, grec,
                                     (rec_here || may_query) ? &vi : nullptr, training ? (1 << 30) : W.term_depth,
                                     &queried, spread ? &sp : nullptr);
        if (spread) aux = make_int4(__float_as_int(sp.thr), __float_as_int(sp.sum), __float_as_int(sp.pdf), aux.w);
        want_q = queried;
        want_r = !queried && rec_here && (vi.kind == MT_LAMBERTIAN || vi.kind == MT_ISOTROPIC);
      }
      if (cont) depth++;
    }
    // warp-wide appends (every lane takes part in the ballots)
    if (MODE == 1) {
      const unsigned ps = warp_append(new_rec, W.pend_count);
      if (new_rec && ps < W.rec_cap) {
        float4 *q = W.pend + 5 * (size_t)ps;
        q[0] = make_float4(grec.x.x, grec.x.y, grec.x.z, 0.f);
        q[1] = make_float4(grec.n.x, grec.n.y, grec.n.z, 0.f);
        q[2] = make_float4(grec.d.x, grec.d.y, grec.d.z, 0.f);
        q[3] = make_float4(grec.T.x, grec.T.y, grec.T.z, 0.f);
        q[4] = make_float4(grec.L.x, grec.L.y, grec.L.z, 0.f);
        aux.x = (int)ps;
      }
    } else {
      const unsigned qs = warp_append(want_q, W.q_count);
      if (want_q && qs < W.q_cap) {
        float4 *q = W.queries + 6 * (size_t)qs;
        q[0] = make_float4(vi.p.x, vi.p.y, vi.p.z, vi.rough);
        q[1] = make_float4(vi.wo.x, vi.wo.y, vi.wo.z, 0.f);
        q[2] = make_float4(vi.n.x, vi.n.y, vi.n.z, 0.f);
        q[3] = make_float4(vi.albedo.x, vi.albedo.y, vi.albedo.z, 0.f);
        q[4] = make_float4(Tb.x, Tb.y, Tb.z, __int_as_float((int)pixel));
      }
      const unsigned rs = warp_append(want_r, W.rec_count);
      if (want_r) {
        if (rs < W.rec_cap) {
          float4 *q = W.records + 5 * (size_t)rs;
          q[0] = make_float4(vi.p.x, vi.p.y, vi.p.z, vi.rough);
          q[1] = make_float4(vi.wo.x, vi.wo.y, vi.wo.z, 0.f);
          q[2] = make_float4(vi.n.x, vi.n.y, vi.n.z, 0.f);
          q[3] = make_float4(vi.albedo.x, vi.albedo.y, vi.albedo.z, 0.f);
          q[4] = make_float4(0.f, 0.f, 0.f, 0.f);
          W.pend[2 * (size_t)rs] = make_float4(Tb.x, Tb.y, Tb.z, 0.f);
          W.pend[2 * (size_t)rs + 1] = make_float4(Lb.x, Lb.y, Lb.z, 0.f);
        }
        const int slot = rs < W.rec_cap ? (int)rs : -1;
        if ((aux.w & AUX_COUNT) == 0) aux.x = slot;
        else if ((aux.w & AUX_COUNT) == 1) aux.y = slot;
        else aux.z = slot;
        aux.w++;
      }
    }
    // finished paths: accumulate, complete their records
    const bool ended = live && !cont;
    bool emit_rec = false;
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0;
    if (ended) {
      accumulate(F, pixel, L);
      const float3 Lf = de_nan(L);
      if (MODE == 1 && aux.x >= 0 && aux.x < (int)W.rec_cap) {
        const float4 *q = W.pend + 5 * (size_t)aux.x;
        const float4 qT = q[3], qL = q[4];
        const float3 c = v3((L.x - qL.x) / qT.x, (L.y - qL.y) / qT.y, (L.z - qL.z) / qT.z);
        float wgt = (c.x + c.y + c.z) * (1.f / 3.f);
        if (!(wgt >= 0.f) || !(wgt < 1e6f)) wgt = 0.f;
        const float4 x = q[0];
        r0 = make_float4(x.x, x.y, x.z, wgt);
        r1 = q[1];
        r2 = q[2];
        emit_rec = true;
      }
      if (MODE == 2) {
        const int slots[3] = {aux.x, aux.y, aux.z};
        for (int j = 0; j < (aux.w & AUX_COUNT) && j < 3; j++) {
          const int sl = slots[j];
          if (sl < 0) continue;
          const float4 pT = W.pend[2 * (size_t)sl], pL = W.pend[2 * (size_t)sl + 1];
          float3 tg = v3((Lf.x - pL.x) / pT.x, (Lf.y - pL.y) / pT.y, (Lf.z - pL.z) / pT.z);
          tg = v3(isfinite(tg.x) ? fmaxf(tg.x, 0.f) : 0.f, isfinite(tg.y) ? fmaxf(tg.y, 0.f) : 0.f,
                  isfinite(tg.z) ? fmaxf(tg.z, 0.f) : 0.f);
          W.records[5 * (size_t)sl + 4] = make_float4(tg.x, tg.y, tg.z, 1.f);
        }
      }
    }
    if (MODE == 1) {
      const unsigned rs = warp_append(emit_rec, W.rec_count) % W.rec_cap;  // ring: the newest records win
      if (emit_rec) {
        W.records[3 * (size_t)rs] = r0;
        W.records[3 * (size_t)rs + 1] = r1;
        W.records[3 * (size_t)rs + 2] = r2;
      }
    }
    // regenerate finished paths from the global sample counter
    unsigned long long base;
    int rank;
    warp_claim(ended, &C->issued, base, rank);
    bool fresh = false;
    if (ended) {
      const unsigned long long s = base + (unsigned long long)rank;
      if (s < F.total) {
        int i, j;
        sample_coords(F, s + W.sample_offset, pixel, sample, i, j);
        sample += W.sample_add;
        r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, cfg.key);
        depth = 0;
        T = v3(1.f, 1.f, 1.f);
        L = v3(0.f, 0.f, 0.f);
        aux = fresh_aux(F, W, pixel, sample);
        fresh = true;
      }
    }
    const bool emit = cont || fresh;
    const unsigned slot = warp_append(emit, &C->count[cur ^ 1]);
    if (emit) {
      write_path(out, slot, r, depth, T, L, pixel, sample);
      store_aux<MODE>(out, slot, aux);
    }
  }
}

// Persistent engine: every lane carries one path in registers; when its
// path ends it accumulates and claims the next camera sample (one atomic per
// warp for all lanes that need one), so lanes do not idle behind the longest
// path of their warp.
template <int MIN_BLOCKS, int FEAT = FEAT_ALL>
__global__ void __launch_bounds__(128, MIN_BLOCKS) k_persistent(DevScene S, RenderCfg cfg, FrameDesc F, WfCounters *C) {
  extern __shared__ int2 stack_smem[];
  int2 *stk = stack_smem + threadIdx.x;
  int e = 0;
  unsigned long long segs = 0;
  bool alive = false, done = false;
  Ray r{};
  float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
  uint32_t pixel = 0, sample = 0;
  int depth = 0;
  for (;;) {
    const bool want = !alive && !done;
    if (refill_now(want, alive, cfg.refill)) {
      unsigned long long base;
      int rank;
      warp_claim(want, &C->issued, base, rank);
      if (want) {
        const unsigned long long s = base + (unsigned long long)rank;
        if (s < F.total) {
          int i, j;
          sample_coords(F, s, pixel, sample, i, j);
          r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, cfg.key);
          T = v3(1.f, 1.f, 1.f);
          L = v3(0.f, 0.f, 0.f);
          depth = 0;
          alive = true;
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    if (alive) {
      MediumRng m{make_uint4(pixel, sample, (uint32_t)depth, 0u), cfg.key, 1};
      HitRef h;
      const bool hit = trace_closest<FEAT, FEAT != FEAT_ALL>(S, r, 0.001f, stk, blockDim.x, m, h, e);
      segs++;
      if (shade_vertex(S, cfg, r, hit, h, T, L, depth, pixel, sample)) {
        depth++;
      } else {
        accumulate(F, pixel, L);
        alive = false;
      }
    }
  }
  if (segs) atomicAdd(&C->segments, segs);
  if (e) atomicExch(&C->err, e);
}

// Batched persistent engine: the samples of all items form one sequence
// (prefix sums `first`, kept in shared memory); a claimed sample is mapped
// to its item by binary search and traced in that item's scene.  Warps claim
// consecutive samples, so a warp's lanes nearly always share a scene.
struct BatchItem {
  DevScene scene;
  FrameDesc frame;
  unsigned long long first;
};

template <int MIN_BLOCKS, int FEAT = FEAT_ALL>
__global__ void __launch_bounds__(128, MIN_BLOCKS)
    k_persistent_batch(const BatchItem *__restrict__ items, int n_items, unsigned long long total_all, RenderCfg cfg,
                       WfCounters *C) {
  extern __shared__ int2 stack_smem[];
  __shared__ unsigned long long s_first[TPT_MAX_BATCH];
  for (int i = threadIdx.x; i < n_items; i += blockDim.x) s_first[i] = items[i].first;
  __syncthreads();
  int2 *stk = stack_smem + threadIdx.x;
  int e = 0;
  unsigned long long segs = 0;
  bool alive = false, done = false;
  Ray r{};
  float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
  uint32_t pixel = 0, sample = 0;
  int depth = 0, item = 0;
  for (;;) {
    const bool want = !alive && !done;
    if (refill_now(want, alive, cfg.refill)) {
      unsigned long long base;
      int rank;
      warp_claim(want, &C->issued, base, rank);
      if (want) {
        const unsigned long long s = base + (unsigned long long)rank;
        if (s < total_all) {
          int lo = 0, hi = n_items - 1;  // last item with first <= s
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_first[mid] <= s) lo = mid; else hi = mid - 1;
          }
          item = lo;
          const BatchItem &B = items[item];
          int i, j;
          sample_coords(B.frame, s - s_first[item], pixel, sample, i, j);
          r = camera_ray(B.scene.cam, i, j, B.frame.nx, B.frame.ny, pixel, sample, cfg.key);
          T = v3(1.f, 1.f, 1.f);
          L = v3(0.f, 0.f, 0.f);
          depth = 0;
          alive = true;
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    if (alive) {
      const DevScene &S = items[item].scene;
      MediumRng m{make_uint4(pixel, sample, (uint32_t)depth, 0u), cfg.key, 1};
      HitRef h;
      const bool hit = trace_closest<FEAT>(S, r, 0.001f, stk, blockDim.x, m, h, e);
      segs++;
      if (shade_vertex(S, cfg, r, hit, h, T, L, depth, pixel, sample)) {
        depth++;
      } else {
        accumulate(items[item].frame, pixel, L);
        alive = false;
      }
    }
  }
  if (segs) atomicAdd(&C->segments, segs);
  if (e) atomicExch(&C->err, e);
}

// Batched persistent engine for sphere-only scenes, with the BVH walk split
// into steps.  In k_persistent_batch a lane traces a whole segment inside one
// call, so a warp runs the walk as long as its longest lane and the others
// idle (4.7 of 32 lanes per instruction on the 64-scene batch).  Here every
// lane keeps its walk's state (stack depth, best hit) in registers: each
// round the traversing lanes advance up to STEP_NODES nodes, and a lane
// whose walk ends waits; once at least `cfg.refill` lanes of the warp wait
// (or none is walking), they shade together, continue or finish their paths,
// claim new camera samples, and start their next walks.  The walk visits the
// same nodes with the same tests, pruning and tie order as trace_closest's
// stack walk (a node's children: boxes by the slab test, sphere leaves by the
// reference's quadratic, inline in the node's record), so every segment
// finds the same closest hit; the shading arithmetic is the same source, but
// the compiler contracts multiply-adds differently in each kernel, so a
// sample's radiance can differ in the last bits (and, where such a bit flips
// a scatter decision, the rest of that path).  A scene that is not one
// top-level BVH item takes trace_closest for its segments.
enum { STEP_NODES = 6 };
enum { LANE_IDLE = 0, LANE_WALK = 1, LANE_READY = 2, LANE_DONE = 3 };

template <int MIN_BLOCKS>
__global__ void __launch_bounds__(128, MIN_BLOCKS)
    k_persistent_batch_step(const BatchItem *__restrict__ items, int n_items, unsigned long long total_all,
                            RenderCfg cfg, WfCounters *C) {
  extern __shared__ int2 stack_smem[];
  __shared__ unsigned long long s_first[TPT_MAX_BATCH];
  for (int i = threadIdx.x; i < n_items; i += blockDim.x) s_first[i] = items[i].first;
  __syncthreads();
  int2 *stk = stack_smem + threadIdx.x;
  const int stride = blockDim.x;
  const float tmin = 0.001f, tmax = 3.402823466e38f;
  int e = 0;
  unsigned long long segs = 0;
  int state = LANE_IDLE;
  Ray r{};
  RayPre W{};
  float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
  uint32_t pixel = 0, sample = 0;
  int depth = 0, item = 0;
  // walk state
  int sp = 0, bl = -1;
  float bt = CUDART_INF_F;
  const f4 *kids = nullptr;
  const int never_pruned = __float_as_int(-CUDART_INF_F);
  const int threshold = cfg.refill < 1 ? 1 : (cfg.refill > 32 ? 32 : cfg.refill);
  for (;;) {
    const unsigned waiting = __ballot_sync(0xffffffffu, state == LANE_IDLE || state == LANE_READY);
    const unsigned walking = __ballot_sync(0xffffffffu, state == LANE_WALK);
    if (waiting && ((int)__popc(waiting) >= threshold || !walking)) {
      // ---- shade the finished walks; continue or finish the paths
      bool start = false;
      if (state == LANE_READY) {
        const DevScene &S = items[item].scene;
        const HitRef h{bt, bl, -1, -1};
        if (shade_vertex(S, cfg, r, bl >= 0, h, T, L, depth, pixel, sample)) {
          depth++;
          start = true;
        } else {
          accumulate(items[item].frame, pixel, L);
          state = LANE_IDLE;
        }
      }
      // ---- idle lanes claim the next camera samples (one atomic per warp)
      const bool want = state == LANE_IDLE;
      unsigned long long base;
      int rank;
      warp_claim(want, &C->issued, base, rank);
      if (want) {
        const unsigned long long sidx = base + (unsigned long long)rank;
        if (sidx < total_all) {
          int lo = 0, hi = n_items - 1;  // last item with first <= sidx
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_first[mid] <= sidx) lo = mid; else hi = mid - 1;
          }
          item = lo;
          const BatchItem &B = items[item];
          int i, j;
          sample_coords(B.frame, sidx - s_first[item], pixel, sample, i, j);
          r = camera_ray(B.scene.cam, i, j, B.frame.nx, B.frame.ny, pixel, sample, cfg.key);
          T = v3(1.f, 1.f, 1.f);
          L = v3(0.f, 0.f, 0.f);
          depth = 0;
          start = true;
        } else {
          state = LANE_DONE;
        }
      }
      // ---- start the next walk: the root box, or the whole segment by
      // trace_closest where the scene is not one top-level BVH
      if (start) {
        segs++;
        const DevScene &S = items[item].scene;
        const int2 it0 = *reinterpret_cast<const int2 *>(S.items);
        bt = CUDART_INF_F;
        bl = -1;
        sp = 0;
        if (S.n_items == 1 && it0.x == ITEM_BVH) {
          W = precompute(r);
          kids = S.node_kids;
          float en;
          const f4 rlo = ldg4(S.node_lo + it0.y), rhi = ldg4(S.node_hi + it0.y);
          if (slab(W, rlo, rhi, tmin, tmax, en)) {
            stk[0] = make_int2(it0.y, never_pruned);
            sp = 1;
          }
          state = sp ? LANE_WALK : LANE_READY;
        } else {
          MediumRng m{make_uint4(pixel, sample, (uint32_t)depth, 0u), cfg.key, 1};
          HitRef h;
          const bool hit = trace_closest<FEAT_SPHERES>(S, r, tmin, stk, stride, m, h, e);
          bt = h.t;
          bl = hit ? h.leaf : -1;
          state = LANE_READY;
        }
      }
    }
    if (__all_sync(0xffffffffu, state == LANE_DONE)) break;
    // ---- walk: up to STEP_NODES nodes per lane (the stack walk of trace_closest)
#pragma unroll 1
    for (int k = 0; k < STEP_NODES && state == LANE_WALK; k++) {
      const int2 en = stk[(sp - 1) * stride];
      --sp;
      if (!(__int_as_float(en.y) > bt)) {
        const f4 *kid = kids + 4 * (size_t)en.x;
        const f4 k0 = ldg4(kid), k1 = ldg4(kid + 1), k2 = ldg4(kid + 2), k3 = ldg4(kid + 3);
        const int left = __float_as_int(k0.w), right = __float_as_int(k2.w);
        int2 q[2];
        float ent[2];
        int nq = 0;
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const int ref = c == 0 ? left : right;
          if (c == 1 && right == left) break;  // n == 1 node: left_ == right_
          if (ref >= 0) {
            float entry;
            const f4 clo = c == 0 ? k0 : k2, chi = c == 0 ? k1 : k3;
            if (slab(W, clo, chi, tmin, tmax, entry)) {
              ent[nq] = entry;
              q[nq++] = make_int2(ref, __float_as_int(prune_key_ext(W, chi.w, entry)));
            }
          } else {  // a sphere leaf, carried in the child's slot
            const f4 sc = c == 0 ? k0 : k2;
            const int leaf = ~ref;
            float t;
            if (sphere_t(v3(sc.x, sc.y, sc.z), (c == 0 ? k1 : k3).x, r, tmin, tmax, t) &&
                (t < bt || (t == bt && leaf > bl))) {  // ties: the larger leaf order (hitable.cc:71)
              bt = t;
              bl = leaf;
            }
          }
        }
        if (nq == 2 && ent[1] > ent[0]) {
          const int2 tq = q[0];
          q[0] = q[1];
          q[1] = tq;
        }
        for (int k2i = 0; k2i < nq; k2i++) {
          if (sp >= TRAVERSAL_STACK) {
            e = TPT_ERR_STACK_OVERFLOW;
          } else {
            stk[sp * stride] = q[k2i];
            sp++;
          }
        }
      }
      if (sp == 0) state = LANE_READY;
    }
  }
  if (segs) atomicAdd(&C->segments, segs);
  if (e) atomicExch(&C->err, e);
}

// Guided persistent engine: as k_persistent, with guided diffuse vertices
// and one training record per recorded path (every `rec_stride`-th sample).
// A recording path parks the state of its first diffuse vertex in `pend`
// (5 float4 per slot) and emits the finished record into the ring when it
// ends, so non-recording lanes carry no record state in registers.
template <int MIN_BLOCKS>
__global__ void __launch_bounds__(128, MIN_BLOCKS)
    k_persistent_guided(DevScene S, RenderCfg cfg, FrameDesc F, WfCounters *C, GuideView gv, uint32_t sample_base,
                        float4 *__restrict__ records, unsigned *rec_count, unsigned rec_cap, uint32_t rec_stride,
                        float4 *__restrict__ pend, unsigned *pend_count) {
  extern __shared__ int2 stack_smem[];
  int2 *stk = stack_smem + threadIdx.x;
  int e = 0;
  unsigned long long segs = 0;
  bool alive = false, done = false;
  Ray r{};
  float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
  uint32_t pixel = 0, sample = 0;
  int depth = 0;
  bool want_rec = false;
  int ps = -1;  // pending-record slot of this path
  for (;;) {
    const bool want = !alive && !done;
    if (refill_now(want, alive, cfg.refill)) {
      unsigned long long base;
      int rank;
      warp_claim(want, &C->issued, base, rank);
      if (want) {
        const unsigned long long s = base + (unsigned long long)rank;
        if (s < F.total) {
          int i, j;
          sample_coords(F, s, pixel, sample, i, j);
          sample += sample_base;
          r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, cfg.key);
          T = v3(1.f, 1.f, 1.f);
          L = v3(0.f, 0.f, 0.f);
          depth = 0;
          want_rec = (s % rec_stride) == 0;
          ps = -1;
          alive = true;
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    bool new_rec = false, ended = false;
    GuideRec rec{};
    if (alive) {
      MediumRng m{make_uint4(pixel, sample, (uint32_t)depth, 0u), cfg.key, 1};
      HitRef h;
      const bool hit = trace_closest(S, r, 0.001f, stk, blockDim.x, m, h, e);
      segs++;
      rec.valid = !want_rec || ps >= 0;  // only a recording path without a record takes one
      if (shade_vertex_t<true>(S, cfg, r, hit, h, T, L, depth, pixel, sample, gv, rec)) {
        depth++;
      } else {
        accumulate(F, pixel, L);
        alive = false;
        ended = true;
      }
      // a NaN direction (the reference's sphere cone sampling from inside
      // the sphere) or position would poison a whole training batch
      new_rec = want_rec && ps < 0 && rec.valid && finite3(rec.x) && finite3(rec.n) && finite3(rec.d);
    }
    const unsigned np = warp_append(new_rec, pend_count);
    if (new_rec && np < rec_cap) {
      float4 *q = pend + 5 * (size_t)np;
      q[0] = make_float4(rec.x.x, rec.x.y, rec.x.z, 0.f);
      q[1] = make_float4(rec.n.x, rec.n.y, rec.n.z, 0.f);
      q[2] = make_float4(rec.d.x, rec.d.y, rec.d.z, 0.f);
      q[3] = make_float4(rec.T.x, rec.T.y, rec.T.z, 0.f);
      q[4] = make_float4(rec.L.x, rec.L.y, rec.L.z, 0.f);
      ps = (int)np;
    }
    bool emit = false;
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0;
    if (ended && ps >= 0) {  // contribution of the sampled direction: (L_final - L_k) / T_k
      const float4 *q = pend + 5 * (size_t)ps;
      const float4 qT = q[3], qL = q[4];
      const float3 c = v3((L.x - qL.x) / qT.x, (L.y - qL.y) / qT.y, (L.z - qL.z) / qT.z);
      float wgt = (c.x + c.y + c.z) * (1.f / 3.f);
      if (!(wgt >= 0.f) || !(wgt < 1e6f)) wgt = 0.f;
      const float4 x = q[0];
      r0 = make_float4(x.x, x.y, x.z, wgt);
      r1 = q[1];
      r2 = q[2];
      emit = true;
      ps = -1;
    }
    const unsigned slot = warp_append(emit, rec_count) % rec_cap;  // ring: the newest records win
    if (emit) {
      records[3 * (size_t)slot] = r0;
      records[3 * (size_t)slot + 1] = r1;
      records[3 * (size_t)slot + 2] = r2;
    }
  }
  if (segs) atomicAdd(&C->segments, segs);
  if (e) atomicExch(&C->err, e);
}

// Radiance-cache engine.  Paths stop at their first diffuse vertex at or
// past `term_depth` and leave a query; every `train_stride`-th path is traced
// to full depth and records its first three diffuse vertices (features now;
// T_k, L_k parked in `pend` under the record's slot; target (L_final - L_k) /
// T_k at its end).
template <int MIN_BLOCKS>
__global__ void __launch_bounds__(128, MIN_BLOCKS)
    k_persistent_nrc(DevScene S, RenderCfg cfg, FrameDesc F, WfCounters *C, unsigned long long sample_offset,
                     int term_depth, uint32_t train_stride, float4 *__restrict__ records, unsigned *rec_count,
                     unsigned rec_cap, float4 *__restrict__ queries, unsigned *q_count, unsigned q_cap,
                     float4 *__restrict__ pend, float spread_sqrt_c) {
  extern __shared__ int2 stack_smem[];
  int2 *stk = stack_smem + threadIdx.x;
  int e = 0;
  unsigned long long segs = 0;
  bool alive = false, done = false, training = false;
  Ray r{};
  float3 T = v3(0.f, 0.f, 0.f), L = v3(0.f, 0.f, 0.f);
  uint32_t pixel = 0, sample = 0;
  int depth = 0;
  int4 rslot = make_int4(-1, -1, -1, 0);  // record slots, count in .w
  Spread sp{};
  GuideView gv{};
  GuideRec grec{};
  for (;;) {
    const bool want = !alive && !done;
    if (refill_now(want, alive, cfg.refill)) {
      unsigned long long base;
      int rank;
      warp_claim(want, &C->issued, base, rank);
      if (want) {
        const unsigned long long s = base + (unsigned long long)rank;
        if (s < F.total) {
          int i, j;
          sample_coords(F, s + sample_offset, pixel, sample, i, j);
          r = camera_ray(S.cam, i, j, F.nx, F.ny, pixel, sample, cfg.key);
          T = v3(1.f, 1.f, 1.f);
          L = v3(0.f, 0.f, 0.f);
          depth = 0;
          training = ((s + sample_offset) % train_stride) == 0;
          rslot = make_int4(-1, -1, -1, 0);
          sp = Spread{spread_sqrt_c, 0.f, 0.f};
          alive = true;
        } else {
          done = true;
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    bool want_q = false, want_r = false;
    VertexInfo vi{};
    float3 qT = T, Tb = T, Lb = L;
    if (alive) {
      MediumRng m{make_uint4(pixel, sample, (uint32_t)depth, 0u), cfg.key, 1};
      HitRef h;
      const bool hit = trace_closest(S, r, 0.001f, stk, blockDim.x, m, h, e);
      segs++;
      const bool spread = !training && spread_sqrt_c > 0.f;
      const bool may_query = !training && (depth >= term_depth || spread);
      const bool rec_here = training && hit && rslot.w < 3;
      bool queried = false;
      const bool cont = shade_vertex_t<false>(S, cfg, r, hit, h, T, L, depth, pixel, sample, gv, grec,
                                              (rec_here || may_query) ? &vi : nullptr,
                                              training ? (1 << 30) : term_depth, &queried, spread ? &sp : nullptr);
      if (queried) {  // ends at a diffuse vertex: the cache adds T x radiance
        want_q = true;
        accumulate(F, pixel, L);
        alive = false;
      } else {
        // records only where queries happen: diffuse vertices
        want_r = rec_here && (vi.kind == MT_LAMBERTIAN || vi.kind == MT_ISOTROPIC);
        if (cont) {
          depth++;
        } else {
          accumulate(F, pixel, L);
          alive = false;
        }
      }
    }
    const unsigned qs = warp_append(want_q, q_count);
    if (want_q && qs < q_cap) {
      float4 *q = queries + 6 * (size_t)qs;
      q[0] = make_float4(vi.p.x, vi.p.y, vi.p.z, vi.rough);
      q[1] = make_float4(vi.wo.x, vi.wo.y, vi.wo.z, 0.f);
      q[2] = make_float4(vi.n.x, vi.n.y, vi.n.z, 0.f);
      q[3] = make_float4(vi.albedo.x, vi.albedo.y, vi.albedo.z, 0.f);
      q[4] = make_float4(qT.x, qT.y, qT.z, __int_as_float((int)pixel));
    }
    const unsigned rs = warp_append(want_r, rec_count);
    if (want_r) {
      const int sl = rs < rec_cap ? (int)rs : -1;
      if (sl >= 0) {
        float4 *q = records + 5 * (size_t)sl;
        q[0] = make_float4(vi.p.x, vi.p.y, vi.p.z, vi.rough);
        q[1] = make_float4(vi.wo.x, vi.wo.y, vi.wo.z, 0.f);
        q[2] = make_float4(vi.n.x, vi.n.y, vi.n.z, 0.f);
        q[3] = make_float4(vi.albedo.x, vi.albedo.y, vi.albedo.z, 0.f);
        q[4] = make_float4(0.f, 0.f, 0.f, 0.f);
        pend[2 * (size_t)sl] = make_float4(Tb.x, Tb.y, Tb.z, 0.f);
        pend[2 * (size_t)sl + 1] = make_float4(Lb.x, Lb.y, Lb.z, 0.f);
      }
      if (rslot.w == 0) rslot.x = sl;
      else if (rslot.w == 1) rslot.y = sl;
      else rslot.z = sl;
      rslot.w++;
    }
    if (training && !alive && rslot.w > 0) {  // path finished: targets of its records
      const float3 Lf = de_nan(L);
      const int slots[3] = {rslot.x, rslot.y, rslot.z};
      for (int k = 0; k < rslot.w && k < 3; k++) {
        if (slots[k] < 0) continue;
        const float4 pT = pend[2 * (size_t)slots[k]], pL = pend[2 * (size_t)slots[k] + 1];
        float3 tg = v3((Lf.x - pL.x) / pT.x, (Lf.y - pL.y) / pT.y, (Lf.z - pL.z) / pT.z);
        tg = v3(isfinite(tg.x) ? fmaxf(tg.x, 0.f) : 0.f, isfinite(tg.y) ? fmaxf(tg.y, 0.f) : 0.f,
                isfinite(tg.z) ? fmaxf(tg.z, 0.f) : 0.f);
        records[5 * (size_t)slots[k] + 4] = make_float4(tg.x, tg.y, tg.z, 1.f);
      }
      rslot = make_int4(-1, -1, -1, 0);
    }
  }
  if (segs) atomicAdd(&C->segments, segs);
  if (e) atomicExch(&C->err, e);
}

// mean = sum / spp, image order (row 0 = top).
__global__ void k_resolve(FrameDesc F, float *__restrict__ out) {
  const long long npix = (long long)F.nx * F.ny;
  const float inv = 1.0f / (float)F.spp;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
    if (F.accum64) {
      const double d = (double)F.spp;
      out[3 * p] = (float)(F.accum64[3 * p] / d);
      out[3 * p + 1] = (float)(F.accum64[3 * p + 1] / d);
      out[3 * p + 2] = (float)(F.accum64[3 * p + 2] / d);
    } else {
      const float4 a = F.accum[p];
      out[3 * p] = a.x * inv;
      out[3 * p + 1] = a.y * inv;
      out[3 * p + 2] = a.z * inv;
    }
  }
}

}  // namespace tpt

using namespace tpt;

// ============================================================== context ===
namespace {

struct Slot {
  void *arena = nullptr;
  size_t bytes = 0;
  DevScene ds{};
  bool live = false;
  bool tuned = false;        // tpt_autotune result for engine = AUTO
  tpt_render_params tp{};
  int cache_engine = 0;      // tpt_autotune_nrc result for cached renders (0: none),
  int cache_block = 128, cache_variant = 4;  // and its persistent launch shape
  float world_lo[3] = {0, 0, 0}, world_hi[3] = {0, 0, 0};
};

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct tpt_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own = nullptr;
  int sm_count = 0;
  std::vector<Slot> slots;
  DevBuf path[2], path_aux[2], hits, accum, accum64, staging, rays, hitf, hiti;
  DevBuf learn_pend;  // wavefront learned renders: pending record state
  DevBuf batch_table, batch_accum, batch_staging;
  DevBuf guide_table, guide_records, guide_count;
  long long guide_last_count = 0;  // records of the last guided pass
  GuideNet *guide = nullptr;
  DevBuf nrc_records, nrc_queries, nrc_counts;
  CacheNet *cache = nullptr;
  cudaGraphExec_t batch_graph = nullptr;  // replayed while the batch key matches
  uint64_t batch_key = 0;
  WfCounters *counters = nullptr;       // device
  WfCounters *counters_host = nullptr;  // pinned
  int *err = nullptr;                   // device error flag for trace
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t prof_ev[24] = {};  // per-launch timing of one graph (8 iterations x 3)
  int flat_nodes = DEFAULT_FLAT_MAX;
};

static thread_local char g_last_error[256] = "";

static tpt_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return TPT_OK;
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return TPT_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TPT_ERR_NO_DEVICE;
  return TPT_ERR_CUDA;
}
#define TPT_CUDA(x)                              \
  do {                                           \
    cudaError_t e_ = (x);                        \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

static tpt_status ensure(DevBuf &b, size_t bytes) {
  if (b.bytes >= bytes) return TPT_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  TPT_CUDA(cudaMalloc(&b.p, bytes));
  b.bytes = bytes;
  return TPT_OK;
}

static int stack_smem(int block) { return block * TRAVERSAL_STACK * (int)sizeof(int2); }

// Dynamic shared memory above 48 KB needs the per-kernel opt-in.
template <class K>
static cudaError_t smem_optin(K kernel, int smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

template <class K>
static int grid_for(const tpt_context *ctx, K kernel, int block, int smem) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (per_sm < 1) per_sm = 1;
  return ctx->sm_count * per_sm;
}

extern "C" {

const char *tpt_last_error(void) { return g_last_error; }

tpt_status tpt_context_create(int32_t device, tpt_context **out) {
  if (!out) return TPT_ERR_INVALID_ARGUMENT;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return TPT_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(device));
  auto *c = new (std::nothrow) tpt_context();
  if (!c) return TPT_ERR_OUT_OF_MEMORY;
  c->device = device;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->counters, sizeof(WfCounters));
  if (e == cudaSuccess) e = cudaMallocHost(&c->counters_host, sizeof(WfCounters));
  if (e == cudaSuccess) e = cudaMalloc(&c->err, sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e != cudaSuccess) {
    tpt_context_destroy(c);
    return cuda_status(e);
  }
  c->stream = c->own;
  *out = c;
  return TPT_OK;
}

void tpt_context_destroy(tpt_context *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto &s : c->slots)
    if (s.arena) cudaFree(s.arena);
  DevBuf *bufs[] = {&c->path[0], &c->path[1], &c->hits,        &c->accum,       &c->accum64,      &c->staging,
                    &c->rays,    &c->hitf,    &c->hiti,        &c->batch_table, &c->batch_accum, &c->batch_staging};
  for (DevBuf *b : bufs)
    if (b->p) cudaFree(b->p);
  if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
  DevBuf *gb[] = {&c->guide_table, &c->guide_records, &c->guide_count, &c->nrc_records, &c->nrc_queries,
                  &c->nrc_counts, &c->path_aux[0], &c->path_aux[1], &c->learn_pend};
  for (DevBuf *b : gb)
    if (b->p) cudaFree(b->p);
  guide_destroy(c->guide);
  cache_destroy(c->cache);
  if (c->counters) cudaFree(c->counters);
  if (c->counters_host) cudaFreeHost(c->counters_host);
  if (c->err) cudaFree(c->err);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (auto &ev : c->prof_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
}

tpt_status tpt_context_set_stream(tpt_context *c, void *stream) {
  if (!c) return TPT_ERR_INVALID_ARGUMENT;
  c->stream = stream ? (cudaStream_t)stream : c->own;
  return TPT_OK;
}

tpt_status tpt_context_set_option(tpt_context *c, int32_t option, int64_t value) {
  if (!c) return TPT_ERR_INVALID_ARGUMENT;
  if (option == TPT_OPT_FLAT_NODES) {
    if (value < 0 || value > (1ll << 30)) return TPT_ERR_INVALID_ARGUMENT;
    c->flat_nodes = (int)value;
    return TPT_OK;
  }
  return TPT_ERR_INVALID_ARGUMENT;
}

// Device view of a scene whose arena (layout L) starts at `base`.
static DevScene dev_scene_at(const HostScene &S, const ArenaLayout &L, uint8_t *base) {
  DevScene d{};
  d.node_lo = (const f4 *)(base + L.off[0]);
  d.node_hi = (const f4 *)(base + L.off[1]);
  d.node_skip = (const int32_t *)(base + L.off[2]);
  d.leaf_hdr = (const i4 *)(base + L.off[3]);
  d.leaf_user = (const int32_t *)(base + L.off[4]);
  d.leaf_data = (const f4 *)(base + L.off[5]);
  d.items = (const i2 *)(base + L.off[6]);
  d.mat_i = (const i4 *)(base + L.off[7]);
  d.mat_f = (const f4 *)(base + L.off[8]);
  d.tex_i = (const i4 *)(base + L.off[9]);
  d.tex_f = (const f4 *)(base + L.off[10]);
  d.images = base + L.off[11];
  d.perlin_grad = (const f4 *)(base + L.off[12]);
  d.perlin_perm = (const int32_t *)(base + L.off[13]);
  d.light_i = (const i4 *)(base + L.off[14]);
  d.light_f = (const f4 *)(base + L.off[15]);
  d.node_kids = (const f4 *)(base + L.off[16]);
  d.flat_max = DEFAULT_FLAT_MAX;
  bool only_spheres = true, media = false;
  for (const i4 &h : S.leaf_hdr) {
    const int t = h.x & LEAF_TYPE_MASK;
    only_spheres = only_spheres && t == LT_SPHERE;
    media = media || t == LT_MEDIUM || t == LT_MSPHERE;
  }
  d.feat = only_spheres ? FEAT_SPHERES : (media ? FEAT_ALL : FEAT_NO_MEDIA);
  d.n_nodes = (int32_t)S.node_lo.size();
  d.n_leaves = (int32_t)S.leaf_hdr.size();
  d.n_items = (int32_t)S.items.size();
  d.n_mats = (int32_t)S.mat_i.size();
  d.n_texs = (int32_t)S.tex_i.size();
  d.n_lights = (int32_t)S.light_i.size();
  d.light_is_list = S.light_is_list;
  d.has_lights = S.has_lights;
  d.cam = S.cam;
  return d;
}

// The LBVH build jobs of a scene whose arena starts at `base` (device).
static LbvhArgs lbvh_args(const HostScene &S, const ArenaLayout &L, uint8_t *base) {
  LbvhArgs a;
  a.jobs = (const i4 *)(base + L.off[ARENA_LBVH_JOBS]);
  a.n_jobs = (int32_t)S.lbvh_jobs.size();
  a.prims = (const f4 *)(base + L.off[ARENA_LBVH_PRIMS]);
  a.n_prims = (int32_t)(S.lbvh_prims.size() / 2);
  a.n_keys = S.lbvh_keys;
  a.max_pad = S.lbvh_max_pad;
  a.node_lo = (f4 *)(base + L.off[0]);
  a.node_hi = (f4 *)(base + L.off[1]);
  a.node_skip = (int32_t *)(base + L.off[2]);
  a.node_kids = (f4 *)(base + L.off[16]);
  a.n_leaves = (int32_t)S.leaf_hdr.size();
  a.leaf_hdr = (const i4 *)(base + L.off[3]);
  a.leaf_data = (const f4 *)(base + L.off[5]);
  a.work = base + L.off[ARENA_LBVH_WORK];
  return a;
}

// Builds a TPT_BVH_LBVH scene's trees in its device arena, waits for the
// build and checks it: every reference inside its tree, and the traversal
// stack bound against the trees' depths (the compile-time check counted each
// tree as one level).
static tpt_status lbvh_scene_build(const HostScene &S, const ArenaLayout &L, uint8_t *base, cudaStream_t stream) {
  if (S.lbvh_jobs.empty()) return TPT_OK;
  const LbvhArgs a = lbvh_args(S, L, base);
  TPT_CUDA(lbvh_build(a, stream));
  std::vector<int32_t> depth(a.n_jobs + 1);
  TPT_CUDA(cudaMemcpyAsync(depth.data(), lbvh_depths(a.work, a.n_prims, a.n_jobs, a.n_keys),
                           sizeof(int32_t) * (a.n_jobs + 1), cudaMemcpyDeviceToHost, stream));
  TPT_CUDA(cudaStreamSynchronize(stream));
  if (depth[a.n_jobs]) {
    std::snprintf(g_last_error, sizeof(g_last_error), "LBVH build produced %d nodes with out-of-range references",
                  depth[a.n_jobs]);
    return TPT_ERR_CUDA;
  }
  int top = 0, blas = 0;
  for (int j = 0; j < a.n_jobs; j++) {
    int &d = S.lbvh_blas[j] ? blas : top;
    d = std::max(d, depth[j]);
  }
  const int need = top + 2 + (S.n_blas ? blas + 2 : 0);  // as the host compiler counts it
  if (need > TRAVERSAL_STACK) {
    std::snprintf(g_last_error, sizeof(g_last_error),
                  "LBVH of depth %d (instanced %d) needs %d traversal stack entries, the device has %d", top, blas,
                  need, (int)TRAVERSAL_STACK);
    return TPT_ERR_STACK_OVERFLOW;
  }
  return TPT_OK;
}

tpt_status tpt_scene_upload(tpt_context *c, const tpt_scene *sc, int32_t *slot) {
  if (!c || !sc || !slot) return TPT_ERR_INVALID_ARGUMENT;
  const HostScene &S = *host_scene(sc);
  TPT_CUDA(cudaSetDevice(c->device));
  const ArenaLayout L = arena_layout(S);
  std::vector<uint8_t> host(L.total, 0);
  ArenaSection sec[ARENA_SECTIONS];
  arena_sections(S, sec);
  for (int i = 0; i < ARENA_SECTIONS; i++)
    if (sec[i].bytes && sec[i].data) std::memcpy(host.data() + L.off[i], sec[i].data, sec[i].bytes);
  Slot s;
  TPT_CUDA(cudaMalloc(&s.arena, L.total));
  cudaError_t e = cudaMemcpyAsync(s.arena, host.data(), L.total, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    cudaFree(s.arena);
    return cuda_status(e);
  }
  s.bytes = L.total;
  uint8_t *base = (uint8_t *)s.arena;
  const tpt_status bst = lbvh_scene_build(S, L, base, c->stream);
  if (bst != TPT_OK) {
    cudaStreamSynchronize(c->stream);
    cudaFree(s.arena);
    return bst;
  }
  s.ds = dev_scene_at(S, L, base);
  for (int i = 0; i < 3; i++) {
    s.world_lo[i] = S.world_lo[i];
    s.world_hi[i] = S.world_hi[i];
  }
  s.live = true;
  for (size_t i = 0; i < c->slots.size(); i++)
    if (!c->slots[i].live) {
      c->slots[i] = s;
      *slot = (int32_t)i;
      return TPT_OK;
    }
  c->slots.push_back(s);
  *slot = (int32_t)c->slots.size() - 1;
  return TPT_OK;
}

tpt_status tpt_bvh_build_boxes(tpt_context *c, const float *boxes, int32_t n, float *node_boxes,
                               int32_t *node_kids, int32_t *node_skip, int32_t *depth) {
  if (!c || !boxes || n < 1 || !node_boxes || !node_kids || !node_skip || !depth) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  const int m = n > 1 ? n - 1 : 1;
  const int64_t pad = lbvh_pad(n);
  // one job: inputs, the node arrays of m nodes and the build scratch
  const size_t sz[7] = {sizeof(i4), 2 * (size_t)n * sizeof(f4), (size_t)m * sizeof(f4), (size_t)m * sizeof(f4),
                        4 * (size_t)m * sizeof(f4), (size_t)m * sizeof(int32_t), lbvh_work_bytes(n, 1, pad)};
  size_t off[7], total = 0;
  for (int i = 0; i < 7; i++) {
    off[i] = total;
    total += lbvh_align(sz[i]);
  }
  std::vector<uint8_t> host(off[2], 0);
  const i4 job{0, n, 0, 0};
  std::memcpy(host.data(), &job, sizeof job);
  f4 *prims = (f4 *)(host.data() + off[1]);
  for (int i = 0; i < n; i++) {
    const int32_t ref = ~i, zero = 0;
    prims[2 * i] = f4{boxes[6 * i], boxes[6 * i + 1], boxes[6 * i + 2], 0};
    prims[2 * i + 1] = f4{boxes[6 * i + 3], boxes[6 * i + 4], boxes[6 * i + 5], 0};
    std::memcpy(&prims[2 * i].w, &ref, 4);
    std::memcpy(&prims[2 * i + 1].w, &zero, 4);
  }
  uint8_t *d = nullptr;
  TPT_CUDA(cudaMalloc(&d, total));
  LbvhArgs a;
  a.jobs = (const i4 *)d;
  a.n_jobs = 1;
  a.prims = (const f4 *)(d + off[1]);
  a.n_prims = n;
  a.n_keys = pad;
  a.max_pad = (int32_t)pad;
  a.node_lo = (f4 *)(d + off[2]);
  a.node_hi = (f4 *)(d + off[3]);
  a.node_kids = (f4 *)(d + off[4]);
  a.node_skip = (int32_t *)(d + off[5]);
  a.n_leaves = n;
  a.leaf_hdr = nullptr;  // boxes only
  a.leaf_data = nullptr;
  a.work = d + off[6];
  std::vector<f4> lo(m), hi(m);
  cudaError_t e = cudaMemcpyAsync(d, host.data(), off[2], cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = lbvh_build(a, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(lo.data(), a.node_lo, m * sizeof(f4), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hi.data(), a.node_hi, m * sizeof(f4), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(node_skip, a.node_skip, m * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  int32_t dep[2] = {0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dep, lbvh_depths(a.work, n, 1, pad), sizeof dep, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_status(e);
  if (dep[1]) {
    std::snprintf(g_last_error, sizeof(g_last_error), "LBVH build produced %d nodes with out-of-range references",
                  dep[1]);
    return TPT_ERR_CUDA;
  }
  *depth = dep[0];
  for (int p = 0; p < m; p++) {
    const float b[6] = {lo[p].x, lo[p].y, lo[p].z, hi[p].x, hi[p].y, hi[p].z};
    std::memcpy(node_boxes + 6 * (size_t)p, b, sizeof b);
    std::memcpy(node_kids + 2 * (size_t)p, &lo[p].w, 4);
    std::memcpy(node_kids + 2 * (size_t)p + 1, &hi[p].w, 4);
  }
  return TPT_OK;
}

tpt_status tpt_scene_release(tpt_context *c, int32_t slot) {
  if (!c || slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  cudaStreamSynchronize(c->stream);
  cudaFree(c->slots[slot].arena);
  c->slots[slot] = Slot{};
  if (c->batch_graph) {  // its table may point at the released arena
    cudaGraphExecDestroy(c->batch_graph);
    c->batch_graph = nullptr;
    c->batch_key = 0;
  }
  return TPT_OK;
}

tpt_status tpt_trace_closest(tpt_context *c, int32_t slot, const float *rays, int64_t n, uint64_t seed, float *hit_f,
                             int32_t *hit_i, int32_t mem) {
  if (!c || n < 0 || (n > 0 && (!rays || !hit_f || !hit_i))) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  if (n == 0) return TPT_OK;
  TPT_CUDA(cudaSetDevice(c->device));
  const float *d_rays = rays;
  float *d_f = hit_f;
  int *d_i = hit_i;
  if (mem == TPT_MEM_HOST) {
    tpt_status st;
    if ((st = ensure(c->rays, (size_t)n * 7 * sizeof(float))) != TPT_OK) return st;
    if ((st = ensure(c->hitf, (size_t)n * 9 * sizeof(float))) != TPT_OK) return st;
    if ((st = ensure(c->hiti, (size_t)n * 2 * sizeof(int))) != TPT_OK) return st;
    TPT_CUDA(cudaMemcpyAsync(c->rays.p, rays, (size_t)n * 7 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    d_rays = (const float *)c->rays.p;
    d_f = (float *)c->hitf.p;
    d_i = (int *)c->hiti.p;
  }
  TPT_CUDA(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
  const int block = 128, smem = stack_smem(block);
  DevScene ds = c->slots[slot].ds;
  ds.flat_max = c->flat_nodes;
  // the same specialisation the renders of this scene use
  auto kern = ds.feat == FEAT_SPHERES   ? k_trace_closest<FEAT_SPHERES>
              : ds.feat == FEAT_NO_MEDIA ? k_trace_closest<FEAT_NO_MEDIA>
                                         : k_trace_closest<FEAT_ALL>;
  int grid = grid_for(c, kern, block, smem);
  const long long need = (n + block - 1) / block;
  if (grid > need) grid = (int)need;
  kern<<<grid, block, smem, c->stream>>>(ds, d_rays, n, make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)), d_f, d_i,
                                         c->err);
  TPT_CUDA(cudaGetLastError());
  int herr = 0;
  TPT_CUDA(cudaMemcpyAsync(&herr, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  if (mem == TPT_MEM_HOST) {
    TPT_CUDA(cudaMemcpyAsync(hit_f, d_f, (size_t)n * 9 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    TPT_CUDA(cudaMemcpyAsync(hit_i, d_i, (size_t)n * 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  }
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  return herr ? (tpt_status)herr : TPT_OK;
}

void tpt_render_params_default(tpt_render_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->width = 400;   // main.cpp:31-40 defaults
  p->height = 200;
  p->spp = 10;
  p->max_depth = 50;
  p->semantics = TPT_SEMANTICS_REFERENCE;
  p->background = TPT_BACKGROUND_BLACK;
  p->sky_scale = 1.0f;
  p->seed = 1;
}

}  // extern "C"

static PathBuf path_view(DevBuf &b, size_t wave, DevBuf *aux = nullptr) {
  float4 *base = (float4 *)b.p;
  return PathBuf{base, base + wave, base + 2 * wave, base + 3 * wave, aux ? (int4 *)aux->p : nullptr};
}

// Wavefront render; returns after all samples are accumulated.  MODE 0: the
// plain tracer; 1 / 2: a pass of the guided / cached renderer (W).
template <int MODE>
static tpt_status run_wavefront_t(tpt_context *c, const DevScene &S, const RenderCfg &cfg, const FrameDesc &F,
                                  int block, size_t wave, bool profile, tpt_render_stats *stats,
                                  const WfLearn *W = nullptr) {
  tpt_status st;
  if ((st = ensure(c->path[0], wave * 4 * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->path[1], wave * 4 * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->hits, wave * sizeof(int4))) != TPT_OK) return st;
  if (MODE > 0) {
    if ((st = ensure(c->path_aux[0], wave * sizeof(int4))) != TPT_OK) return st;
    if ((st = ensure(c->path_aux[1], wave * sizeof(int4))) != TPT_OK) return st;
  }
  PathBuf P[2] = {path_view(c->path[0], wave, MODE > 0 ? &c->path_aux[0] : nullptr),
                  path_view(c->path[1], wave, MODE > 0 ? &c->path_aux[1] : nullptr)};
  const unsigned first = (unsigned)std::min<unsigned long long>(wave, F.total);
  WfCounters init{};
  init.count[0] = first;
  init.issued = first;
  std::memcpy(c->counters_host, &init, sizeof(init));
  TPT_CUDA(cudaMemcpyAsync(c->counters, c->counters_host, sizeof(WfCounters), cudaMemcpyHostToDevice, c->stream));
  const int smem = stack_smem(block);
  auto traverse = S.feat == FEAT_SPHERES   ? k_wf_traverse<FEAT_SPHERES>
                  : S.feat == FEAT_NO_MEDIA ? k_wf_traverse<FEAT_NO_MEDIA>
                                            : k_wf_traverse<FEAT_ALL>;
  TPT_CUDA(smem_optin(traverse, smem));
  const int g_gen = std::max(1, std::min<int>((int)((first + block - 1) / block), c->sm_count * 8));
  if constexpr (MODE == 0)
    k_wf_generate<<<g_gen, block, 0, c->stream>>>(S, F, P[0], 0ull, first, cfg.key);
  else
    k_wf_generate_learn<MODE == 0 ? 1 : MODE><<<g_gen, block, 0, c->stream>>>(S, F, P[0], first, cfg.key, *W);
  TPT_CUDA(cudaGetLastError());
  int launches = 1;
  const int g_tr = grid_for(c, traverse, block, smem);
  const int g_sh = MODE == 0 ? grid_for(c, k_wf_shade, block, 0) : grid_for(c, k_wf_shade_learn<MODE == 0 ? 1 : MODE>, block, 0);
  // iteration bound: every sample lives at most max_depth+1 segments
  const unsigned long long max_iters = (F.total * (unsigned long long)(cfg.max_depth + 1)) / wave + 64;
  // capture an even number of iterations (buffer parity returns) as a graph;
  // with profiling, event-record nodes bracket every launch
  const int kIters = 8;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (profile && !c->prof_ev[0]) {
    for (auto &ev : c->prof_ev)
      if (cudaEventCreate(&ev) != cudaSuccess) return TPT_ERR_CUDA;
  }
  TPT_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int it = 0; it < kIters; it++) {
    const int cur = it & 1;
    if (profile) cudaEventRecordWithFlags(c->prof_ev[3 * it], c->stream, cudaEventRecordExternal);
    traverse<<<g_tr, block, smem, c->stream>>>(S, P[cur], cur, c->counters, (int4 *)c->hits.p, cfg.key);
    if (profile) cudaEventRecordWithFlags(c->prof_ev[3 * it + 1], c->stream, cudaEventRecordExternal);
    if constexpr (MODE == 0)
      k_wf_shade<<<g_sh, block, 0, c->stream>>>(S, cfg, F, P[cur], P[cur ^ 1], cur, c->counters,
                                                (const int4 *)c->hits.p);
    else
      k_wf_shade_learn<MODE><<<g_sh, block, 0, c->stream>>>(S, cfg, F, P[cur], P[cur ^ 1], cur, c->counters,
                                                            (const int4 *)c->hits.p, *W);
    if (profile) cudaEventRecordWithFlags(c->prof_ev[3 * it + 2], c->stream, cudaEventRecordExternal);
  }
  cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_status(e);
  unsigned long long iters = 0;
  tpt_status result = TPT_OK;
  for (;;) {
    e = cudaGraphLaunch(exec, c->stream);
    if (e != cudaSuccess) { result = cuda_status(e); break; }
    launches += 2 * kIters;
    iters += kIters;
    e = cudaMemcpyAsync(c->counters_host, c->counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { result = cuda_status(e); break; }
    const WfCounters &h = *c->counters_host;
    if (profile && stats) {
      for (int it = 0; it < kIters; it++) {
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, c->prof_ev[3 * it], c->prof_ev[3 * it + 1]);
        cudaEventElapsedTime(&b, c->prof_ev[3 * it + 1], c->prof_ev[3 * it + 2]);
        stats->traverse_ms += a;
        stats->shade_ms += b;
      }
      stats->traverse_launches += kIters;
      stats->shade_launches += kIters;
    }
    if (h.err) { result = h.err; break; }
    if (h.count[0] == 0 && h.issued >= F.total) break;
    if (iters > max_iters) { result = TPT_ERR_DEVICE_TIMEOUT; break; }
  }
  cudaGraphExecDestroy(exec);
  if (stats) {
    stats->iterations = (int32_t)iters;
    stats->kernel_launches += launches;
    stats->segments = (int64_t)c->counters_host->segments;
  }
  return result;
}

static tpt_status run_wavefront(tpt_context *c, const DevScene &S, const RenderCfg &cfg, const FrameDesc &F, int block,
                                size_t wave, bool profile, tpt_render_stats *stats) {
  return run_wavefront_t<0>(c, S, cfg, F, block, wave, profile, stats);
}

// Register-capped variants of the persistent kernel (occupancy vs spills),
// selected by tpt_render_params.wave when the persistent engine runs.
typedef void (*PersistentKernel)(DevScene, RenderCfg, FrameDesc, WfCounters *);
static PersistentKernel persistent_variant(int v, int feat = FEAT_ALL) {
  if (feat == FEAT_SPHERES) {  // sphere-only scenes: the traversal without the other leaf kinds
    switch (v) {
      case 5: return k_persistent<5, FEAT_SPHERES>;
      case 6: return k_persistent<6, FEAT_SPHERES>;
      default: return k_persistent<4, FEAT_SPHERES>;
    }
  }
  // scenes without media keep the general persistent kernel: its no-media
  // specialisation measured slower on the Cornell box (950 against 1036
  // Msamples/s: different register allocation), unlike the wavefront traversal
  switch (v) {
    case 5: return k_persistent<5>;
    case 6: return k_persistent<6>;
    case 8: return k_persistent<8>;
    default: return k_persistent<4>;
  }
}

// Samples [begin, F.total) of the frame (sample-major order: sample index
// s covers pixel s % npix, sample s / npix).
static tpt_status run_persistent(tpt_context *c, const DevScene &S, const RenderCfg &cfg, const FrameDesc &F, int block,
                                 int variant, bool profile, tpt_render_stats *stats,
                                 unsigned long long begin = 0) {
  WfCounters init{};
  init.issued = begin;
  std::memcpy(c->counters_host, &init, sizeof(init));
  TPT_CUDA(cudaMemcpyAsync(c->counters, c->counters_host, sizeof(WfCounters), cudaMemcpyHostToDevice, c->stream));
  const int smem = stack_smem(block);
  const PersistentKernel kern = persistent_variant(variant, S.feat);
  if (block > 128) return TPT_ERR_INVALID_ARGUMENT;  // launch bounds of the variants
  TPT_CUDA(smem_optin(kern, smem));
  const int grid = grid_for(c, kern, block, smem);
  if (profile && !c->prof_ev[0]) {
    for (auto &ev : c->prof_ev)
      if (cudaEventCreate(&ev) != cudaSuccess) return TPT_ERR_CUDA;
  }
  if (profile) cudaEventRecord(c->prof_ev[0], c->stream);
  kern<<<grid, block, smem, c->stream>>>(S, cfg, F, c->counters);
  TPT_CUDA(cudaGetLastError());
  if (profile) cudaEventRecord(c->prof_ev[1], c->stream);
  TPT_CUDA(cudaMemcpyAsync(c->counters_host, c->counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, c->stream));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) {
    stats->iterations = 1;
    stats->kernel_launches += 1;
    stats->segments = (int64_t)c->counters_host->segments;
    if (profile) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->prof_ev[0], c->prof_ev[1]);
      stats->traverse_ms = ms;  // traversal and shading are fused in this engine
      stats->traverse_launches = 1;
    }
  }
  return c->counters_host->err ? (tpt_status)c->counters_host->err : TPT_OK;
}

extern "C" tpt_status tpt_render(tpt_context *c, int32_t slot, const tpt_render_params *p, float *out_rgb,
                                 int32_t mem, tpt_render_stats *stats) {
  if (!c || !p || !out_rgb) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->max_depth < 0) return TPT_ERR_INVALID_ARGUMENT;
  const unsigned long long npix = (unsigned long long)p->width * p->height;
  const unsigned long long total = npix * (unsigned long long)p->spp;
  if (npix > 0x7fffffffull || (unsigned long long)p->spp > 0x7fffffffull) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  tpt_status st;
  if ((st = ensure(c->accum, npix * sizeof(float4))) != TPT_OK) return st;
  if (p->accumulate_fp64 && (st = ensure(c->accum64, npix * 3 * sizeof(double))) != TPT_OK) return st;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  FrameDesc F{p->width, p->height, p->spp, total, (float4 *)c->accum.p,
              p->accumulate_fp64 ? (double *)c->accum64.p : nullptr};
  RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
  tpt_render_params tuned;
  if (p->engine == TPT_ENGINE_AUTO && c->slots[slot].tuned) {
    tuned = *p;
    tuned.engine = c->slots[slot].tp.engine;
    tuned.block = c->slots[slot].tp.block;
    tuned.wave = c->slots[slot].tp.wave;
    tuned.flat_nodes = c->slots[slot].tp.flat_nodes;
    p = &tuned;
  }
  const int block = p->block > 0 ? p->block : 128;
  if (block % 32 || block > 1024) return TPT_ERR_INVALID_ARGUMENT;
  size_t wave = p->wave > 0 ? (size_t)p->wave : (size_t)1 << 20;
  if (wave > total) wave = (size_t)std::max<unsigned long long>(total, 32ull);
  TPT_CUDA(cudaEventRecord(c->ev0, c->stream));
  TPT_CUDA(cudaMemsetAsync(c->accum.p, 0, npix * sizeof(float4), c->stream));
  if (F.accum64) TPT_CUDA(cudaMemsetAsync(c->accum64.p, 0, npix * 3 * sizeof(double), c->stream));
  DevScene S = c->slots[slot].ds;
  S.flat_max = p->flat_nodes > 0 ? p->flat_nodes : c->flat_nodes;
  const int engine = p->engine == TPT_ENGINE_AUTO ? TPT_ENGINE_PERSISTENT : p->engine;
  if (engine == TPT_ENGINE_PERSISTENT)
    st = run_persistent(c, S, cfg, F, p->block > 0 ? block : 128, p->wave, p->profile != 0, stats);
  else
    st = run_wavefront(c, S, cfg, F, block, wave, p->profile != 0, stats);
  if (st != TPT_OK) return st;
  float *dst = out_rgb;
  if (mem == TPT_MEM_HOST) {
    if ((st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
    dst = (float *)c->staging.p;
  }
  const int rblock = 256;
  const int rgrid = (int)std::min<unsigned long long>((npix + rblock - 1) / rblock, (unsigned long long)c->sm_count * 16);
  k_resolve<<<rgrid, rblock, 0, c->stream>>>(F, dst);
  TPT_CUDA(cudaGetLastError());
  TPT_CUDA(cudaEventRecord(c->ev1, c->stream));
  if (mem == TPT_MEM_HOST)
    TPT_CUDA(cudaMemcpyAsync(out_rgb, dst, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->device_ms = ms;
    stats->samples = (int64_t)total;
    stats->kernel_launches += 1;
  }
  return TPT_OK;
}

// =============================================================== batches ==
static uint64_t fnv1a(uint64_t h, const void *data, size_t n) {
  const uint8_t *b = (const uint8_t *)data;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

typedef void (*BatchKernel)(const BatchItem *, int, unsigned long long, RenderCfg, WfCounters *);
// Register variants 4-6 (and 8): k_persistent_batch; 14-16: the stepped walk
// (k_persistent_batch_step), sphere-only batches only.
static BatchKernel batch_variant(int v, int feat = FEAT_ALL) {
  if (feat == FEAT_SPHERES) {  // every item sphere-only
    switch (v) {
      case 14: return k_persistent_batch_step<4>;
      case 15: return k_persistent_batch_step<5>;
      case 16: return k_persistent_batch_step<6>;
      case 5: return k_persistent_batch<5, FEAT_SPHERES>;
      case 6: return k_persistent_batch<6, FEAT_SPHERES>;
      default: return k_persistent_batch<4, FEAT_SPHERES>;
    }
  }
  switch (v) {
    case 5: return k_persistent_batch<5>;
    case 6: return k_persistent_batch<6>;
    case 8: return k_persistent_batch<8>;
    default: return k_persistent_batch<4>;
  }
}

extern "C" tpt_status tpt_render_snapshots(tpt_context *c, int32_t slot, const tpt_render_params *p,
                                           int32_t bonus_pic, float *out_rgb, float *snapshots_rgb, int32_t mem,
                                           tpt_render_stats *stats) {
  if (!c || !p || !out_rgb || (bonus_pic > 0 && !snapshots_rgb)) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->max_depth < 0 || bonus_pic < 0 || bonus_pic > p->spp)
    return TPT_ERR_INVALID_ARGUMENT;
  const unsigned long long npix = (unsigned long long)p->width * p->height;
  if (npix > 0x7fffffffull) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  tpt_status st;
  if ((st = ensure(c->accum, npix * sizeof(float4))) != TPT_OK) return st;
  if (p->accumulate_fp64 && (st = ensure(c->accum64, npix * 3 * sizeof(double))) != TPT_OK) return st;
  if (mem == TPT_MEM_HOST && (st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  const Slot &sl = c->slots[slot];
  int block = p->block > 0 ? p->block : 128, variant = p->wave;
  if (p->engine == TPT_ENGINE_AUTO && sl.tuned && sl.tp.engine == TPT_ENGINE_PERSISTENT) {
    block = sl.tp.block;
    variant = sl.tp.wave;
  }
  DevScene S = sl.ds;
  S.flat_max = p->flat_nodes > 0 ? p->flat_nodes : (sl.tuned ? sl.tp.flat_nodes : c->flat_nodes);
  const RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                      make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
  TPT_CUDA(cudaMemsetAsync(c->accum.p, 0, npix * sizeof(float4), c->stream));
  if (p->accumulate_fp64) TPT_CUDA(cudaMemsetAsync(c->accum64.p, 0, npix * 3 * sizeof(double), c->stream));
  const int slice = bonus_pic > 0 ? p->spp / bonus_pic : p->spp;
  const int rgrid = (int)std::min<unsigned long long>((npix + 255) / 256, (unsigned long long)c->sm_count * 16);
  // resolves the running mean over the first `spp` samples into host or device image `out`
  auto emit = [&](int spp, float *out) -> tpt_status {
    FrameDesc R{p->width, p->height, spp, npix * (unsigned long long)spp, (float4 *)c->accum.p,
                p->accumulate_fp64 ? (double *)c->accum64.p : nullptr};
    float *dst = mem == TPT_MEM_HOST ? (float *)c->staging.p : out;
    k_resolve<<<rgrid, 256, 0, c->stream>>>(R, dst);
    TPT_CUDA(cudaGetLastError());
    if (mem == TPT_MEM_HOST) {
      TPT_CUDA(cudaMemcpyAsync(out, dst, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
      TPT_CUDA(cudaStreamSynchronize(c->stream));
    }
    return TPT_OK;
  };
  int done = 0;
  for (int k = 0; k <= bonus_pic; k++) {
    const int upto = k < bonus_pic ? (k + 1) * slice : p->spp;
    if (upto > done) {
      FrameDesc F{p->width, p->height, upto, npix * (unsigned long long)upto, (float4 *)c->accum.p,
                  p->accumulate_fp64 ? (double *)c->accum64.p : nullptr};
      tpt_render_stats part{};
      if ((st = run_persistent(c, S, cfg, F, block, variant, false, &part, npix * (unsigned long long)done)) != TPT_OK)
        return st;
      if (stats) {
        stats->segments += part.segments;
        stats->kernel_launches += part.kernel_launches;
        stats->iterations += part.iterations;
      }
      done = upto;
    }
    if ((st = emit(upto, k < bonus_pic ? snapshots_rgb + (size_t)k * npix * 3 : out_rgb)) != TPT_OK) return st;
  }
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) stats->samples = (int64_t)npix * p->spp;
  return TPT_OK;
}

// One share of a frame split across GPUs: samples [begin, end) of every
// pixel, summed into the caller's float4 accumulators.  The persistent
// engine's global sample counter starts at begin * npix, and every sample
// draws from its own (pixel, sample index) stream, so the shares of any
// partition of [0, spp) sum to the accumulators of the whole frame.
extern "C" tpt_status tpt_render_range(tpt_context *c, int32_t slot, const tpt_render_params *p,
                                       int32_t sample_begin, int32_t sample_end, float *accum_dev,
                                       tpt_render_stats *stats) {
  if (!c || !p || !accum_dev) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  if (p->width <= 0 || p->height <= 0 || p->max_depth < 0 || sample_begin < 0 || sample_end < sample_begin)
    return TPT_ERR_INVALID_ARGUMENT;
  if (((uintptr_t)accum_dev & 15) != 0) return TPT_ERR_INVALID_ARGUMENT;  // float4 per pixel
  const unsigned long long npix = (unsigned long long)p->width * p->height;
  if (npix > 0x7fffffffull) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  if (stats) std::memset(stats, 0, sizeof(*stats));
  TPT_CUDA(cudaMemsetAsync(accum_dev, 0, npix * sizeof(float4), c->stream));
  if (sample_end > sample_begin) {
    const Slot &sl = c->slots[slot];
    int block = p->block > 0 ? p->block : 128, variant = p->wave;
    if (p->engine == TPT_ENGINE_AUTO && sl.tuned && sl.tp.engine == TPT_ENGINE_PERSISTENT) {
      block = sl.tp.block;
      variant = sl.tp.wave;
    }
    DevScene S = sl.ds;
    S.flat_max = p->flat_nodes > 0 ? p->flat_nodes : (sl.tuned ? sl.tp.flat_nodes : c->flat_nodes);
    const RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                        make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
    const FrameDesc F{p->width, p->height, sample_end, npix * (unsigned long long)sample_end, (float4 *)accum_dev,
                      nullptr};
    const tpt_status st = run_persistent(c, S, cfg, F, block, variant, p->profile != 0, stats,
                                         npix * (unsigned long long)sample_begin);
    if (st != TPT_OK) return st;
  }
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) stats->samples = (int64_t)npix * (sample_end - sample_begin);
  return TPT_OK;
}

// Mean image from summed float4 accumulators (after the sum across ranks).
extern "C" tpt_status tpt_resolve_sums(tpt_context *c, const float *accum_dev, int32_t width, int32_t height,
                                       int32_t spp, float *out_rgb, int32_t mem) {
  if (!c || !accum_dev || !out_rgb || width <= 0 || height <= 0 || spp <= 0) return TPT_ERR_INVALID_ARGUMENT;
  if (((uintptr_t)accum_dev & 15) != 0 || (mem != TPT_MEM_HOST && mem != TPT_MEM_DEVICE))
    return TPT_ERR_INVALID_ARGUMENT;
  const unsigned long long npix = (unsigned long long)width * height;
  if (npix > 0x7fffffffull) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  tpt_status st;
  if (mem == TPT_MEM_HOST && (st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
  const FrameDesc R{width, height, spp, npix * (unsigned long long)spp, (float4 *)accum_dev, nullptr};
  float *dst = mem == TPT_MEM_HOST ? (float *)c->staging.p : out_rgb;
  const int rgrid = (int)std::min<unsigned long long>((npix + 255) / 256, (unsigned long long)c->sm_count * 16);
  k_resolve<<<rgrid, 256, 0, c->stream>>>(R, dst);
  TPT_CUDA(cudaGetLastError());
  if (mem == TPT_MEM_HOST)
    TPT_CUDA(cudaMemcpyAsync(out_rgb, dst, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  return TPT_OK;
}

extern "C" tpt_status tpt_render_batch(tpt_context *c, const tpt_batch_item *items, int32_t n,
                                       const tpt_render_params *p, int32_t mem, tpt_render_stats *stats) {
  if (!c || !items || !p || n < 1 || n > TPT_MAX_BATCH) return TPT_ERR_INVALID_ARGUMENT;
  const int block = p->block > 0 ? p->block : 128;
  if (block % 32 || block > 128 || p->max_depth < 0) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  std::vector<BatchItem> table(n);
  std::vector<size_t> pix_off(n + 1, 0);
  unsigned long long total = 0;
  for (int k = 0; k < n; k++) {
    const tpt_batch_item &it = items[k];
    if (it.slot < 0 || it.slot >= (int32_t)c->slots.size() || !c->slots[it.slot].live) return TPT_ERR_BAD_HANDLE;
    if (it.width <= 0 || it.height <= 0 || it.spp <= 0 || !it.out_rgb) return TPT_ERR_INVALID_ARGUMENT;
    const unsigned long long npix = (unsigned long long)it.width * it.height;
    if (npix > 0x7fffffffull) return TPT_ERR_INVALID_ARGUMENT;
    pix_off[k + 1] = pix_off[k] + (size_t)npix;
    table[k].first = total;
    total += npix * (unsigned long long)it.spp;
  }
  tpt_status st;
  if ((st = ensure(c->batch_accum, pix_off[n] * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->batch_table, (size_t)n * sizeof(BatchItem))) != TPT_OK) return st;
  if (mem == TPT_MEM_HOST && (st = ensure(c->batch_staging, pix_off[n] * 3 * sizeof(float))) != TPT_OK) return st;
  float4 *acc = (float4 *)c->batch_accum.p;
  for (int k = 0; k < n; k++) {
    const tpt_batch_item &it = items[k];
    table[k].scene = c->slots[it.slot].ds;
    table[k].scene.flat_max = p->flat_nodes > 0 ? p->flat_nodes : c->flat_nodes;
    table[k].frame = FrameDesc{it.width, it.height, it.spp, (unsigned long long)it.width * it.height * it.spp,
                               acc + pix_off[k], nullptr};
  }
  const RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                      make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
  uint64_t key = 1469598103934665603ull;
  key = fnv1a(key, table.data(), table.size() * sizeof(BatchItem));
  key = fnv1a(key, &cfg, sizeof(cfg));
  key = fnv1a(key, &block, sizeof(block));
  key = fnv1a(key, &p->wave, sizeof(p->wave));
  key = fnv1a(key, &mem, sizeof(mem));
  for (int k = 0; k < n; k++) key = fnv1a(key, &items[k].out_rgb, sizeof(float *));
  int feat = FEAT_SPHERES;  // the widest feature set of the items (batch kernels: spheres only or all)
  for (int k = 0; k < n; k++)
    if (table[k].scene.feat != FEAT_SPHERES) feat = FEAT_ALL;
  const BatchKernel kern = batch_variant(p->wave, feat);
  const int smem = stack_smem(block);
  if (!c->batch_graph || c->batch_key != key) {
    if (c->batch_graph) {
      cudaGraphExecDestroy(c->batch_graph);
      c->batch_graph = nullptr;
    }
    TPT_CUDA(cudaMemcpyAsync(c->batch_table.p, table.data(), (size_t)n * sizeof(BatchItem), cudaMemcpyHostToDevice,
                             c->stream));
    TPT_CUDA(cudaStreamSynchronize(c->stream));
    TPT_CUDA(smem_optin(kern, smem));
    const int grid = grid_for(c, kern, block, smem);
    cudaGraph_t graph = nullptr;
    TPT_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(c->batch_accum.p, 0, pix_off[n] * sizeof(float4), c->stream);
    cudaMemsetAsync(c->counters, 0, sizeof(WfCounters), c->stream);
    kern<<<grid, block, smem, c->stream>>>((const BatchItem *)c->batch_table.p, n, total, cfg, c->counters);
    for (int k = 0; k < n; k++) {
      const unsigned long long npix = pix_off[k + 1] - pix_off[k];
      float *dst = mem == TPT_MEM_HOST ? (float *)c->batch_staging.p + 3 * pix_off[k] : items[k].out_rgb;
      const int rgrid = (int)std::min<unsigned long long>((npix + 255) / 256, (unsigned long long)c->sm_count * 8);
      k_resolve<<<rgrid, 256, 0, c->stream>>>(table[k].frame, dst);
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->batch_graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      c->batch_graph = nullptr;
      return cuda_status(e);
    }
    c->batch_key = key;
  }
  TPT_CUDA(cudaEventRecord(c->ev0, c->stream));
  TPT_CUDA(cudaGraphLaunch(c->batch_graph, c->stream));
  TPT_CUDA(cudaEventRecord(c->ev1, c->stream));
  TPT_CUDA(cudaMemcpyAsync(c->counters_host, c->counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, c->stream));
  if (mem == TPT_MEM_HOST)
    for (int k = 0; k < n; k++)
      TPT_CUDA(cudaMemcpyAsync(items[k].out_rgb, (float *)c->batch_staging.p + 3 * pix_off[k],
                               (pix_off[k + 1] - pix_off[k]) * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->device_ms = ms;
    stats->samples = (int64_t)total;
    stats->segments = (int64_t)c->counters_host->segments;
    stats->iterations = 1;
    stats->kernel_launches = 1 + n;
    if (p->profile) {
      stats->traverse_ms = ms;
      stats->traverse_launches = 1;
    }
  }
  return c->counters_host->err ? (tpt_status)c->counters_host->err : TPT_OK;
}

// ============================================================= autotuner ==
extern "C" tpt_status tpt_autotune_batch(tpt_context *c, const tpt_batch_item *items, int32_t n,
                                         tpt_render_params *p, int32_t spp_divisor, double *best_msps) {
  if (!c || !items || !p || n < 1 || n > TPT_MAX_BATCH || spp_divisor < 1) return TPT_ERR_INVALID_ARGUMENT;
  std::vector<tpt_batch_item> probe(items, items + n);
  for (auto &it : probe) it.spp = std::max(1, it.spp / spp_divisor);
  struct Cand {
    int block, variant, flat, refill;
  };
  std::vector<Cand> cands;
  for (int block : {64, 128})
    for (int var : {4, 5, 6})
      for (int flat : {16, 48}) cands.push_back({block, var, flat, 1});
  bool spheres_only = true;
  for (int k = 0; k < n; k++) {
    const tpt_batch_item &it = items[k];
    if (it.slot < 0 || it.slot >= (int32_t)c->slots.size() || !c->slots[it.slot].live) return TPT_ERR_BAD_HANDLE;
    if (c->slots[it.slot].ds.feat != FEAT_SPHERES) spheres_only = false;
  }
  if (spheres_only)  // the stepped walk, and how many lanes wait before they shade
    for (int var : {14, 15})
      for (int refill : {16, 20, 24}) cands.push_back({64, var, 16, refill});
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return cuda_status(ce);
  }
  tpt_status st = TPT_OK;
  // Msamples/s of a candidate: the fastest of `reps` timed runs after the
  // run that captures its graph
  auto measure = [&](const Cand &cd, int reps, double &msps) -> tpt_status {
    tpt_render_params q = *p;
    q.block = cd.block;
    q.wave = cd.variant;
    q.flat_nodes = cd.flat;
    q.refill = cd.refill;
    q.profile = 0;
    tpt_render_stats rs{};
    float best_ms = 1e30f;
    for (int rep = 0; rep <= reps; rep++) {
      float ms = 0.f;
      cudaEventRecord(e0, c->stream);
      const tpt_status s2 = tpt_render_batch(c, probe.data(), n, &q, TPT_MEM_DEVICE, &rs);
      if (s2 != TPT_OK) return s2;
      cudaEventRecord(e1, c->stream);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) best_ms = std::min(best_ms, ms);
    }
    msps = (double)rs.samples / (best_ms * 1e3);
    return TPT_OK;
  };
  std::vector<std::pair<double, int>> ranked;
  for (int i = 0; i < (int)cands.size() && st == TPT_OK; i++) {
    double msps = 0.0;
    st = measure(cands[i], 1, msps);
    ranked.push_back({msps, i});
  }
  // the best three again, fastest of three runs
  double best = -1.0;
  Cand win = cands[0];
  if (st == TPT_OK) {
    std::sort(ranked.begin(), ranked.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
      return a.first > b.first;
    });
    win = cands[ranked[0].second];
    for (int k = 0; k < 3 && k < (int)ranked.size() && st == TPT_OK; k++) {
      double msps = 0.0;
      st = measure(cands[ranked[k].second], 3, msps);
      if (st == TPT_OK && msps > best) {
        best = msps;
        win = cands[ranked[k].second];
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != TPT_OK) return st;
  p->block = win.block;
  p->wave = win.variant;
  p->flat_nodes = win.flat;
  p->refill = win.refill;
  if (best_msps) *best_msps = best;
  return TPT_OK;
}

extern "C" tpt_status tpt_autotune(tpt_context *c, int32_t slot, tpt_render_params *p, int32_t probe_spp,
                                   double *best_msps) {
  if (!c || !p || probe_spp <= 0 || p->width <= 0 || p->height <= 0) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  struct Cand {
    int engine, block, wave, flat;
  };
  std::vector<Cand> cands;
  for (int block : {64, 128})
    for (int var : {4, 5, 6})
      for (int flat : {16, 48, 1 << 20}) cands.push_back({TPT_ENGINE_PERSISTENT, block, var, flat});
  for (int block : {128, 256})
    for (int wave : {1 << 19, 1 << 20}) cands.push_back({TPT_ENGINE_WAVEFRONT, block, wave, 48});
  const size_t npix = (size_t)p->width * p->height;
  // a probe of a few M samples is dominated by the launch tail of the
  // persistent kernels: probe at least 16 M samples
  probe_spp = std::max<int32_t>(probe_spp, (int32_t)((16ull << 20) / npix) + 1);
  tpt_status st;
  if ((st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
  // Msamples/s of a candidate: the fastest of `reps` timed runs after one
  // untimed run (caches, allocations)
  auto measure = [&](const Cand &cd, int spp, int reps, double &msps) -> tpt_status {
    tpt_render_params q = *p;
    q.engine = cd.engine;
    q.block = cd.block;
    q.wave = cd.wave;
    q.flat_nodes = cd.flat;
    q.spp = spp;
    q.profile = 0;
    q.accumulate_fp64 = 0;
    tpt_render_stats rs;
    double t = 1e30;
    for (int rep = 0; rep <= reps; rep++) {
      const tpt_status s2 = tpt_render(c, slot, &q, (float *)c->staging.p, TPT_MEM_DEVICE, &rs);
      if (s2 != TPT_OK) return s2;
      if (rep > 0) t = std::min(t, rs.device_ms);
    }
    msps = (double)npix * spp / (t * 1e3);
    return TPT_OK;
  };
  std::vector<std::pair<double, int>> ranked;
  for (int i = 0; i < (int)cands.size(); i++) {
    double msps = 0.0;
    if ((st = measure(cands[i], probe_spp, 1, msps)) != TPT_OK) return st;
    ranked.push_back({msps, i});
  }
  // the leaders are often within a percent or two, and the launch tail of a
  // short probe hides differences that show on a full frame: time the best
  // three again on a probe of ~0.1 s (at least 4x the first), fastest of
  // three runs
  std::sort(ranked.begin(), ranked.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
    return a.first > b.first;
  });
  const double long_spp = std::ceil(0.1 * ranked[0].first * 1e6 / (double)npix);
  const int refine_spp = (int)std::min<double>(std::max<double>(4.0 * probe_spp, long_spp), 65536.0);
  double best = -1.0;
  Cand win = cands[ranked[0].second];
  for (int k = 0; k < 3 && k < (int)ranked.size(); k++) {
    double msps = 0.0;
    if ((st = measure(cands[ranked[k].second], refine_spp, 3, msps)) != TPT_OK) return st;
    if (msps > best) {
      best = msps;
      win = cands[ranked[k].second];
    }
  }
  p->engine = win.engine;
  p->block = win.block;
  p->wave = win.wave;
  p->flat_nodes = win.flat;
  c->slots[slot].tuned = true;
  c->slots[slot].tp = *p;
  if (best_msps) *best_msps = best;
  return TPT_OK;
}

// ========================================================== path guiding ==
extern "C" void tpt_guide_params_default(tpt_guide_params *g) {
  if (!g) return;
  g->passes = 8;
  g->train_steps = 32;
  g->batch = 16384;
  g->lr = 1e-3f;
  g->grid_res = 16;
  g->alpha = 0.5f;
  g->record_cap = 1 << 20;
  g->seed = 1;
  g->light_share = 0.5f;
  g->warm_start = 0;
}

// Engine of a learned render: as asked, else the slot's tuned one, else the
// wavefront engine (faster than the persistent one in physical semantics on
// the measured scenes: Cornell with the small light 684 vs 570, next week
// 159 vs 98 Msamples/s).
static int learned_engine(const tpt_render_params *p, const Slot &sl) {
  if (p->engine == TPT_ENGINE_WAVEFRONT || p->engine == TPT_ENGINE_PERSISTENT) return p->engine;
  return sl.tuned ? sl.tp.engine : TPT_ENGINE_WAVEFRONT;
}
static size_t wf_wave(const tpt_render_params *p, const Slot &sl) {
  if (p->wave > 0) return (size_t)p->wave;
  if (sl.tuned && sl.tp.engine == TPT_ENGINE_WAVEFRONT && sl.tp.wave > 0) return (size_t)sl.tp.wave;
  return (size_t)1 << 20;
}

extern "C" tpt_status tpt_render_guided(tpt_context *c, int32_t slot, const tpt_render_params *p,
                                        const tpt_guide_params *g, float *out_rgb, int32_t mem,
                                        tpt_render_stats *stats, tpt_guide_stats *gstats) {
  if (!c || !p || !g || !out_rgb) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->max_depth < 0 || g->passes < 1 ||
      p->semantics != TPT_SEMANTICS_PHYSICAL || g->grid_res < 1 || g->grid_res > 64 || g->record_cap < 1 ||
      g->record_cap > (1 << 28) ||
      !(g->alpha >= 0.f && g->alpha <= 1.f) || !(g->light_share >= 0.f && g->light_share <= 1.f) || g->batch < 16)
    return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  const Slot &sl = c->slots[slot];
  const unsigned long long npix = (unsigned long long)p->width * p->height;
  const int spp_pass = (p->spp + g->passes - 1) / g->passes;
  const int spp_total = spp_pass * g->passes;
  tpt_status st;
  // a fresh network for every render (reproducible online training), unless
  // warm_start continues from the context's network
  const bool warm = g->warm_start != 0 && c->guide != nullptr;
  if (!warm) {
    guide_destroy(c->guide);
    c->guide = nullptr;
    if ((st = guide_create(c->device, g->seed, &c->guide)) != TPT_OK) return st;
  }
  const size_t table_f4 = (size_t)g->grid_res * g->grid_res * g->grid_res * 6 * GUIDE_ENTRY;
  if ((st = ensure(c->guide_table, table_f4 * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->guide_records, (size_t)g->record_cap * 3 * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->guide_count, 2 * sizeof(unsigned))) != TPT_OK) return st;  // [0] records, [1] pending
  if ((st = ensure(c->accum, npix * sizeof(float4))) != TPT_OK) return st;
  const float3 lo = make_float3(sl.world_lo[0], sl.world_lo[1], sl.world_lo[2]);
  const float3 ext = make_float3(fmaxf(sl.world_hi[0] - sl.world_lo[0], 1e-6f),
                                 fmaxf(sl.world_hi[1] - sl.world_lo[1], 1e-6f),
                                 fmaxf(sl.world_hi[2] - sl.world_lo[2], 1e-6f));
  DevScene S = sl.ds;
  S.flat_max = p->flat_nodes > 0 ? p->flat_nodes : c->flat_nodes;
  const RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                      make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
  FrameDesc F{p->width, p->height, spp_pass, npix * (unsigned long long)spp_pass, (float4 *)c->accum.p, nullptr};
  // engine: as asked, else the slot's tuned one, else the wavefront (faster in
  // physical semantics on the measured scenes)
  const int engine = learned_engine(p, sl);
  const bool wf = engine == TPT_ENGINE_WAVEFRONT;
  const int block = wf ? (p->block > 0 ? p->block : (sl.tuned && sl.tp.engine == TPT_ENGINE_WAVEFRONT ? sl.tp.block : 128))
                       : 128;
  const size_t wave = wf_wave(p, sl);
  const int smem = stack_smem(block);
  // persistent: the slot's tuned register variant (4 or 5 blocks per SM) and block size
  const bool tuned_p = sl.tuned && sl.tp.engine == TPT_ENGINE_PERSISTENT;
  const int pvar = p->wave > 0 ? p->wave : (tuned_p ? sl.tp.wave : 4);
  const int pblock = p->block > 0 && p->block <= 128 ? p->block : (tuned_p ? sl.tp.block : 128);
  auto kern = pvar == 5 ? k_persistent_guided<5> : k_persistent_guided<4>;
  TPT_CUDA(smem_optin(kern, stack_smem(pblock)));
  const int grid = grid_for(c, kern, pblock, stack_smem(pblock));
  if ((st = ensure(c->learn_pend, (size_t)g->record_cap * 5 * sizeof(float4))) != TPT_OK) return st;
  const unsigned long long per_pass = F.total;
  const uint32_t stride = (uint32_t)std::max<unsigned long long>(1ull, per_pass / (unsigned long long)g->record_cap);
  TPT_CUDA(cudaMemsetAsync(c->accum.p, 0, npix * sizeof(float4), c->stream));
  // records accumulate over the passes in a ring of record_cap entries
  TPT_CUDA(cudaMemsetAsync(c->guide_count.p, 0, sizeof(unsigned), c->stream));
  cudaEvent_t e[4] = {};
  for (auto &ev : e) {
    const cudaError_t ce = cudaEventCreate(&ev);
    if (ce != cudaSuccess) {
      for (auto &x : e)
        if (x) cudaEventDestroy(x);
      return cuda_status(ce);
    }
  }
  double render_ms = 0.0, train_ms = 0.0;
  long long records = 0, segments = 0;
  unsigned emitted_before = 0;
  bool have_table = false;
  tpt_status result = TPT_OK;
  if (warm) {  // the continued network guides from the first pass
    result = guide_refresh(c->guide, g->grid_res, (float4 *)c->guide_table.p, c->stream);
    have_table = result == TPT_OK;
  }
  for (int pass = 0; pass < g->passes && result == TPT_OK; pass++) {
    GuideView gv{have_table ? (const float4 *)c->guide_table.p : nullptr, lo,
                 make_float3(1.f / ext.x, 1.f / ext.y, 1.f / ext.z), g->grid_res, g->alpha, g->light_share};
    cudaEventRecord(e[0], c->stream);
    if (wf) {
      WfLearn W{};
      W.gv = gv;
      W.sample_add = (uint32_t)(pass * spp_pass);
      W.stride = stride;
      W.records = (float4 *)c->guide_records.p;
      W.rec_count = (unsigned *)c->guide_count.p;
      W.rec_cap = (unsigned)g->record_cap;
      W.pend = (float4 *)c->learn_pend.p;
      W.pend_count = (unsigned *)c->guide_count.p + 1;
      cudaMemsetAsync(W.pend_count, 0, sizeof(unsigned), c->stream);
      tpt_render_stats part{};
      result = run_wavefront_t<1>(c, S, cfg, F, block, wave, false, &part, &W);
      if (result != TPT_OK) break;
    } else {
      WfCounters init{};
      std::memcpy(c->counters_host, &init, sizeof(init));
      cudaMemcpyAsync(c->counters, c->counters_host, sizeof(WfCounters), cudaMemcpyHostToDevice, c->stream);
      cudaMemsetAsync((unsigned *)c->guide_count.p + 1, 0, sizeof(unsigned), c->stream);
      kern<<<grid, pblock, stack_smem(pblock), c->stream>>>(
          S, cfg, F, c->counters, gv, (uint32_t)(pass * spp_pass), (float4 *)c->guide_records.p,
          (unsigned *)c->guide_count.p, (unsigned)g->record_cap, stride, (float4 *)c->learn_pend.p,
          (unsigned *)c->guide_count.p + 1);
    }
    cudaEventRecord(e[1], c->stream);
    unsigned count = 0;
    cudaMemcpyAsync(&count, c->guide_count.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t ce = cudaMemcpyAsync(c->counters_host, c->counters, sizeof(WfCounters), cudaMemcpyDeviceToHost,
                                     c->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
    if (ce != cudaSuccess) {
      result = cuda_status(ce);
      break;
    }
    if (c->counters_host->err) {
      result = c->counters_host->err;
      break;
    }
    segments += (long long)c->counters_host->segments;
    records += (unsigned)(count - emitted_before);  // emitted by this pass (counter wraps mod 2^32)
    emitted_before = count;
    count = (unsigned)std::min<long long>(records, g->record_cap);  // held in the ring
    c->guide_last_count = count;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e[0], e[1]);
    render_ms += ms;
    if (pass + 1 < g->passes && count > 0) {
      cudaEventRecord(e[2], c->stream);
      result = guide_train(c->guide, (const float4 *)c->guide_records.p, (int)count, g->train_steps, g->batch, g->lr,
                           lo, ext, g->seed + 7919ull * (pass + 1), c->stream);
      if (result == TPT_OK) result = guide_refresh(c->guide, g->grid_res, (float4 *)c->guide_table.p, c->stream);
      if (result != TPT_OK) break;
      cudaEventRecord(e[3], c->stream);
      if ((ce = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
        result = cuda_status(ce);
        break;
      }
      cudaEventElapsedTime(&ms, e[2], e[3]);
      train_ms += ms;
      have_table = true;
    }
  }
  for (auto &ev : e) cudaEventDestroy(ev);
  if (result != TPT_OK) return result;
  // resolve over all passes
  FrameDesc R = F;
  R.spp = spp_total;
  float *dst = out_rgb;
  if (mem == TPT_MEM_HOST) {
    if ((st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
    dst = (float *)c->staging.p;
  }
  const int rgrid = (int)std::min<unsigned long long>((npix + 255) / 256, (unsigned long long)c->sm_count * 16);
  k_resolve<<<rgrid, 256, 0, c->stream>>>(R, dst);
  TPT_CUDA(cudaGetLastError());
  if (mem == TPT_MEM_HOST)
    TPT_CUDA(cudaMemcpyAsync(out_rgb, dst, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->samples = (int64_t)(npix * (unsigned long long)spp_total);
    stats->segments = segments;
    stats->iterations = g->passes;
    stats->device_ms = render_ms + train_ms;
  }
  if (gstats) {
    gstats->render_ms = render_ms;
    gstats->train_ms = train_ms;
    gstats->final_loss = guide_last_loss(c->guide);
    gstats->records = records;
  }
  return TPT_OK;
}

// ============================================== neural radiance cache =====
extern "C" tpt_status tpt_guide_records(tpt_context *c, float *out, int64_t cap, int64_t *count) {
  if (!c || !count || cap < 0 || (cap > 0 && !out)) return TPT_ERR_INVALID_ARGUMENT;
  *count = c->guide_last_count;
  const long long n = std::min<long long>(cap, c->guide_last_count);
  if (n > 0) {
    TPT_CUDA(cudaSetDevice(c->device));
    TPT_CUDA(cudaMemcpyAsync(out, c->guide_records.p, (size_t)n * 3 * sizeof(float4), cudaMemcpyDeviceToHost,
                             c->stream));
    TPT_CUDA(cudaStreamSynchronize(c->stream));
  }
  return TPT_OK;
}

extern "C" void tpt_nrc_params_default(tpt_nrc_params *n) {
  if (!n) return;
  n->passes = 3;
  n->train_steps = 512;
  n->batch = 16384;
  n->lr = 3e-3f;
  n->terminate_depth = 3;
  n->train_stride = 16;
  n->record_cap = 1 << 20;
  n->query_cap = 1 << 22;
  n->seed = 1;
  n->warm_start = 0;
  n->first_pass_spp = 8;
  n->first_train_steps = 0;
  n->spread_c = 0.01f;
}

extern "C" tpt_status tpt_learned_save(tpt_context *c, int32_t which, float *out, int64_t cap, int64_t *count) {
  if (!c || !count || (which != TPT_NET_GUIDE && which != TPT_NET_CACHE)) return TPT_ERR_INVALID_ARGUMENT;
  tpt_mlp *m = which == TPT_NET_GUIDE ? (c->guide ? guide_mlp(c->guide) : nullptr)
                                      : (c->cache ? cache_mlp(c->cache) : nullptr);
  if (!m) return TPT_ERR_BAD_HANDLE;
  *count = mlp_state_count(m);
  if (!out || cap < *count) return TPT_OK;
  TPT_CUDA(cudaSetDevice(c->device));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  return mlp_save_state(m, out);
}

extern "C" tpt_status tpt_learned_load(tpt_context *c, int32_t which, const float *in, int64_t count) {
  if (!c || !in || (which != TPT_NET_GUIDE && which != TPT_NET_CACHE)) return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  // a context without the network gets one only if the checkpoint fits it
  tpt_status st;
  GuideNet *g = nullptr;
  CacheNet *k = nullptr;
  if (which == TPT_NET_GUIDE && !c->guide && (st = guide_create(c->device, 1, &g)) != TPT_OK) return st;
  if (which == TPT_NET_CACHE && !c->cache && (st = cache_create(c->device, 1, &k)) != TPT_OK) return st;
  tpt_mlp *m = which == TPT_NET_GUIDE ? guide_mlp(g ? g : c->guide) : cache_mlp(k ? k : c->cache);
  st = count == mlp_state_count(m) ? mlp_load_state(m, in) : TPT_ERR_INVALID_ARGUMENT;
  if (st != TPT_OK) {
    guide_destroy(g);
    cache_destroy(k);
    return st;
  }
  if (g) c->guide = g;
  if (k) c->cache = k;
  return TPT_OK;
}

extern "C" tpt_status tpt_render_nrc(tpt_context *c, int32_t slot, const tpt_render_params *p,
                                     const tpt_nrc_params *n, float *out_rgb, int32_t mem, tpt_render_stats *stats,
                                     tpt_nrc_stats *nstats) {
  if (!c || !p || !n || !out_rgb) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->max_depth < 0 || n->passes < 1 ||
      n->terminate_depth < 0 || n->train_stride < 1 || n->record_cap < 16 || n->query_cap < 1024 || n->batch < 16 ||
      n->first_pass_spp < 0 || n->first_train_steps < 0 || !(n->spread_c >= 0.f))
    return TPT_ERR_INVALID_ARGUMENT;
  TPT_CUDA(cudaSetDevice(c->device));
  const Slot &sl = c->slots[slot];
  const unsigned long long npix = (unsigned long long)p->width * p->height;
  tpt_status st;
  // a fresh cache for every render (reproducible online training), unless
  // warm_start continues from the context's cache
  const bool warm = n->warm_start != 0 && c->cache != nullptr;
  // samples per pass: the uncached first pass may have its own size, the
  // other passes share the rest (rounded up, so the frame has >= spp)
  int spp_pass = (p->spp + n->passes - 1) / n->passes;
  int spp_first = spp_pass;
  if (!warm && n->first_pass_spp > 0 && n->passes > 1) {
    spp_first = std::min(n->first_pass_spp, p->spp);
    spp_pass = std::max(1, (p->spp - spp_first + n->passes - 2) / (n->passes - 1));
  }
  const int spp_total = spp_first + spp_pass * (n->passes - 1);
  const float sqrt_c = std::sqrt(n->spread_c);
  if (!warm) {
    cache_destroy(c->cache);
    c->cache = nullptr;
    if ((st = cache_create(c->device, n->seed, &c->cache)) != TPT_OK) return st;
  }
  if ((st = ensure(c->nrc_records, (size_t)n->record_cap * 5 * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->nrc_queries, (size_t)n->query_cap * 6 * sizeof(float4))) != TPT_OK) return st;
  if ((st = ensure(c->nrc_counts, 2 * sizeof(unsigned))) != TPT_OK) return st;
  if ((st = ensure(c->accum, npix * sizeof(float4))) != TPT_OK) return st;
  const float3 lo = make_float3(sl.world_lo[0], sl.world_lo[1], sl.world_lo[2]);
  const float3 ext = make_float3(fmaxf(sl.world_hi[0] - sl.world_lo[0], 1e-6f),
                                 fmaxf(sl.world_hi[1] - sl.world_lo[1], 1e-6f),
                                 fmaxf(sl.world_hi[2] - sl.world_lo[2], 1e-6f));
  DevScene S = sl.ds;
  S.flat_max = p->flat_nodes > 0 ? p->flat_nodes : c->flat_nodes;
  const RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                      make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
  const int engine = p->engine == TPT_ENGINE_AUTO && sl.cache_engine ? sl.cache_engine : learned_engine(p, sl);
  const bool wf = engine == TPT_ENGINE_WAVEFRONT;
  const int wf_block =
      p->block > 0 ? p->block : (sl.tuned && sl.tp.engine == TPT_ENGINE_WAVEFRONT ? sl.tp.block : 128);
  const size_t wave = wf_wave(p, sl);
  // persistent: 64 or 128 threads, 4 or 5 resident blocks per SM (as asked,
  // else the slot's tpt_autotune_nrc choice)
  const bool tuned_c = p->engine == TPT_ENGINE_AUTO && sl.cache_engine == TPT_ENGINE_PERSISTENT;
  const int block = p->block == 64 || p->block == 128 ? p->block : (tuned_c ? sl.cache_block : 128);
  const int variant = p->wave == 4 || p->wave == 5 ? p->wave : (tuned_c ? sl.cache_variant : 4);
  const int smem = stack_smem(block);
  auto kern = variant == 5 ? k_persistent_nrc<5> : k_persistent_nrc<4>;
  TPT_CUDA(smem_optin(kern, smem));
  const int grid = grid_for(c, kern, block, smem);
  if ((st = ensure(c->learn_pend, (size_t)n->record_cap * 2 * sizeof(float4))) != TPT_OK) return st;
  unsigned *counts = (unsigned *)c->nrc_counts.p;  // [0] records, [1] queries
  TPT_CUDA(cudaMemsetAsync(c->accum.p, 0, npix * sizeof(float4), c->stream));
  cudaEvent_t ev[6] = {};
  for (auto &x : ev) {
    const cudaError_t ce = cudaEventCreate(&x);
    if (ce != cudaSuccess) {
      for (auto &y : ev)
        if (y) cudaEventDestroy(y);
      return cuda_status(ce);
    }
  }
  double render_ms = 0, infer_ms = 0, train_ms = 0;
  long long n_rec = 0, n_q = 0, segments = 0;
  FrameDesc F{p->width, p->height, spp_pass, 0, (float4 *)c->accum.p, nullptr};
  const unsigned long long chunk = (unsigned long long)n->query_cap;  // samples per launch
  tpt_status result = TPT_OK;
  for (int pass = 0; pass < n->passes && result == TPT_OK; pass++) {
    const bool cached = pass > 0 || warm;  // a continued cache is queried from the first pass
    const int term = cached ? n->terminate_depth : (1 << 30);
    cudaMemsetAsync(counts, 0, sizeof(unsigned), c->stream);  // records of this pass
    const unsigned long long pass_begin =
        pass == 0 ? 0ull : ((unsigned long long)spp_first + (unsigned long long)(pass - 1) * spp_pass) * npix;
    const unsigned long long pass_total = (unsigned long long)(pass == 0 ? spp_first : spp_pass) * npix;
    for (unsigned long long off = 0; off < pass_total && result == TPT_OK; off += chunk) {
      const unsigned long long cnt = std::min(chunk, pass_total - off);
      FrameDesc Fc = F;
      Fc.total = cnt;
      cudaMemsetAsync(counts + 1, 0, sizeof(unsigned), c->stream);
      cudaEventRecord(ev[0], c->stream);
      if (wf) {
        WfLearn W{};
        W.sample_offset = pass_begin + off;
        W.stride = (uint32_t)n->train_stride;
        W.records = (float4 *)c->nrc_records.p;
        W.rec_count = counts;
        W.rec_cap = (unsigned)n->record_cap;
        W.pend = (float4 *)c->learn_pend.p;
        W.term_depth = term;
        W.spread_sqrt_c = cached ? sqrt_c : 0.f;
        W.queries = (float4 *)c->nrc_queries.p;
        W.q_count = counts + 1;
        W.q_cap = (unsigned)n->query_cap;
        tpt_render_stats part{};
        result = run_wavefront_t<2>(c, S, cfg, Fc, wf_block, wave, false, &part, &W);
        if (result != TPT_OK) break;
      } else {
        WfCounters init{};
        std::memcpy(c->counters_host, &init, sizeof(init));
        cudaMemcpyAsync(c->counters, c->counters_host, sizeof(WfCounters), cudaMemcpyHostToDevice, c->stream);
        kern<<<grid, block, smem, c->stream>>>(S, cfg, Fc, c->counters, pass_begin + off, term,
                                              (uint32_t)n->train_stride, (float4 *)c->nrc_records.p, counts,
                                              (unsigned)n->record_cap, (float4 *)c->nrc_queries.p, counts + 1,
                                              (unsigned)n->query_cap, (float4 *)c->learn_pend.p,
                                              cached ? sqrt_c : 0.f);
      }
      cudaEventRecord(ev[1], c->stream);
      unsigned q = 0;
      cudaMemcpyAsync(&q, counts + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
      cudaError_t ce = cudaMemcpyAsync(c->counters_host, c->counters, sizeof(WfCounters), cudaMemcpyDeviceToHost,
                                       c->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
      if (ce != cudaSuccess) {
        result = cuda_status(ce);
        break;
      }
      if (c->counters_host->err) {
        result = c->counters_host->err;
        break;
      }
      segments += (long long)c->counters_host->segments;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[0], ev[1]);
      render_ms += ms;
      q = std::min<unsigned>(q, (unsigned)n->query_cap);
      n_q += q;
      if (q > 0) {
        cudaEventRecord(ev[2], c->stream);
        result = cache_infer(c->cache, (const float4 *)c->nrc_queries.p, (int)q, lo, ext, F.accum, c->stream);
        if (result != TPT_OK) break;
        cudaEventRecord(ev[3], c->stream);
        if ((ce = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
          result = cuda_status(ce);
          break;
        }
        cudaEventElapsedTime(&ms, ev[2], ev[3]);
        infer_ms += ms;
      }
    }
    if (result != TPT_OK) break;
    unsigned nr = 0;
    cudaError_t ce = cudaMemcpyAsync(&nr, counts, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
    if (ce != cudaSuccess) {
      result = cuda_status(ce);
      break;
    }
    nr = std::min<unsigned>(nr, (unsigned)n->record_cap);
    n_rec += nr;
    if (pass + 1 < n->passes && nr > 0) {
      cudaEventRecord(ev[4], c->stream);
      const int steps = pass == 0 && n->first_train_steps > 0 ? n->first_train_steps : n->train_steps;
      result = cache_train(c->cache, (const float4 *)c->nrc_records.p, (int)nr, steps, n->batch, n->lr, lo,
                           ext, (uint32_t)(n->seed * 2654435761ull + pass), c->stream);
      if (result != TPT_OK) break;
      cudaEventRecord(ev[5], c->stream);
      if ((ce = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
        result = cuda_status(ce);
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[4], ev[5]);
      train_ms += ms;
    }
  }
  for (auto &x : ev) cudaEventDestroy(x);
  if (result == TPT_OK) result = cache_check(c->cache, c->stream);
  if (result != TPT_OK) return result;
  FrameDesc R = F;
  R.spp = spp_total;
  float *dst = out_rgb;
  if (mem == TPT_MEM_HOST) {
    if ((st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
    dst = (float *)c->staging.p;
  }
  const int rgrid = (int)std::min<unsigned long long>((npix + 255) / 256, (unsigned long long)c->sm_count * 16);
  k_resolve<<<rgrid, 256, 0, c->stream>>>(R, dst);
  TPT_CUDA(cudaGetLastError());
  if (mem == TPT_MEM_HOST)
    TPT_CUDA(cudaMemcpyAsync(out_rgb, dst, npix * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  TPT_CUDA(cudaStreamSynchronize(c->stream));
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->samples = (int64_t)(npix * (unsigned long long)spp_total);
    stats->segments = segments;
    stats->iterations = n->passes;
    stats->device_ms = render_ms + infer_ms + train_ms;
  }
  if (nstats) {
    nstats->render_ms = render_ms;
    nstats->infer_ms = infer_ms;
    nstats->train_ms = train_ms;
    nstats->final_loss = cache_last_loss(c->cache);
    nstats->records = n_rec;
    nstats->queries = n_q;
  }
  return TPT_OK;
}

// The engine of the slot's cached renders: the wavefront engine and the
// persistent one at 64 or 128 threads and 4 or 5 resident blocks per SM
// each trace a short cached render (an untrained cache: the paths' lengths
// and the queries do not depend on the weights, and training and inference
// cost the same on every engine); the fastest by render time is kept for
// TPT_ENGINE_AUTO.
extern "C" tpt_status tpt_autotune_nrc(tpt_context *c, int32_t slot, const tpt_render_params *p, int32_t probe_spp,
                                       int32_t *engine_out) {
  if (!c || !p || probe_spp < 2 || p->width <= 0 || p->height <= 0) return TPT_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot >= (int32_t)c->slots.size() || !c->slots[slot].live) return TPT_ERR_BAD_HANDLE;
  tpt_nrc_params n;
  tpt_nrc_params_default(&n);
  n.passes = 2;
  n.first_pass_spp = 1;
  n.train_steps = 0;
  const size_t npix = (size_t)p->width * p->height;
  tpt_status st;
  if ((st = ensure(c->staging, npix * 3 * sizeof(float))) != TPT_OK) return st;
  struct Cand {
    int engine, block, variant;
  };
  const Cand cands[] = {{TPT_ENGINE_WAVEFRONT, 0, 0},  {TPT_ENGINE_PERSISTENT, 64, 4}, {TPT_ENGINE_PERSISTENT, 64, 5},
                        {TPT_ENGINE_PERSISTENT, 128, 4}, {TPT_ENGINE_PERSISTENT, 128, 5}};
  Cand best = cands[0];
  double best_ms = 1e30;
  for (const Cand &cd : cands) {
    tpt_render_params q = *p;
    q.engine = cd.engine;
    q.block = cd.block;   // wavefront: 0 = the slot's tuned block and queue
    q.wave = cd.variant;
    q.spp = probe_spp;
    q.profile = 0;
    q.accumulate_fp64 = 0;
    double ms = 1e30;
    for (int rep = 0; rep < 3; rep++) {  // the first run warms caches and allocations
      tpt_nrc_stats ns;
      if ((st = tpt_render_nrc(c, slot, &q, &n, (float *)c->staging.p, TPT_MEM_DEVICE, nullptr, &ns)) != TPT_OK)
        return st;
      if (rep > 0) ms = std::min(ms, ns.render_ms);
    }
    if (ms < best_ms) {
      best_ms = ms;
      best = cd;
    }
  }
  Slot &sl = c->slots[slot];
  sl.cache_engine = best.engine;
  if (best.engine == TPT_ENGINE_PERSISTENT) {
    sl.cache_block = best.block;
    sl.cache_variant = best.variant;
  }
  if (engine_out) *engine_out = best.engine;
  return TPT_OK;
}

// ======================================================= no-allocation path
// Scratch of tpt_render_noalloc: float4 accumulators for up to
// TPT_NOALLOC_MAX_PIXELS pixels, then the counters.  Host code must not use
// the symbol as an address: its device address comes from
// cudaGetSymbolAddress, looked up once per device.
static constexpr size_t kNoallocAccumBytes = (size_t)TPT_NOALLOC_MAX_PIXELS * sizeof(float4);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocAccumBytes + 256];

static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[64];  // per device ordinal

static tpt_status noalloc_scratch(int device, void **out) {
  if (device < 0 || device >= 64) return TPT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void *addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    g_noalloc_addr[device] = addr;
  }
  *out = g_noalloc_addr[device];
  return TPT_OK;
}

extern "C" tpt_status tpt_render_noalloc(const tpt_scene *scene, void *arena_dev, int64_t arena_bytes,
                                         const tpt_render_params *p, float *out_rgb_dev, void *stream_ptr) {
  auto invalid = [](const char *why) {
    std::snprintf(g_last_error, sizeof(g_last_error), "tpt_render_noalloc: %s", why);
    return TPT_ERR_INVALID_ARGUMENT;
  };
  if (!scene || !arena_dev || !p || !out_rgb_dev) return invalid("scene, arena, params and output must be non-NULL");
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->max_depth < 0)
    return invalid("width, height and spp must be positive and max_depth non-negative");
  if (p->accumulate_fp64)
    return invalid("accumulate_fp64 is not supported (the scratch holds FP32 accumulators only)");
  const unsigned long long npix = (unsigned long long)p->width * (unsigned long long)p->height;
  if (npix > (unsigned long long)TPT_NOALLOC_MAX_PIXELS) {
    std::snprintf(g_last_error, sizeof(g_last_error),
                  "tpt_render_noalloc: %llu pixels exceed TPT_NOALLOC_MAX_PIXELS (%d)", npix,
                  TPT_NOALLOC_MAX_PIXELS);
    return TPT_ERR_INVALID_ARGUMENT;
  }
  const HostScene &H = *host_scene(scene);
  const ArenaLayout L = arena_layout(H);
  if (arena_bytes < (int64_t)L.total) {
    std::snprintf(g_last_error, sizeof(g_last_error), "tpt_render_noalloc: arena buffer of %lld bytes, need %zu",
                  (long long)arena_bytes, L.total);
    return TPT_ERR_INVALID_ARGUMENT;
  }
  const int block = p->block > 0 ? p->block : 128;
  if (block % 32 || block > 128) return invalid("block must be a multiple of 32 and at most 128");
  cudaStream_t stream = (cudaStream_t)stream_ptr;
  int device = 0;
  TPT_CUDA(cudaGetDevice(&device));
  void *scratch = nullptr;
  tpt_status st = noalloc_scratch(device, &scratch);
  if (st == TPT_ERR_INVALID_ARGUMENT) return invalid("device ordinal out of range (0..63)");
  if (st != TPT_OK) return st;
  int sm_count = 0;
  TPT_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));

  // the scene: section by section from the host vectors into the caller's buffer
  ArenaSection sec[ARENA_SECTIONS];
  arena_sections(H, sec);
  uint8_t *base = (uint8_t *)arena_dev;
  for (int i = 0; i < ARENA_SECTIONS; i++)
    if (sec[i].bytes && sec[i].data)
      TPT_CUDA(cudaMemcpyAsync(base + L.off[i], sec[i].data, sec[i].bytes, cudaMemcpyHostToDevice, stream));
  {  // TPT_BVH_LBVH: the trees are built in the caller's buffer on every call
    const tpt_status bst = lbvh_scene_build(H, L, base, stream);
    if (bst != TPT_OK) return bst;
  }
  DevScene d = dev_scene_at(H, L, base);
  d.flat_max = p->flat_nodes > 0 ? p->flat_nodes : DEFAULT_FLAT_MAX;

  // the scratch keeps the previous call's contents: clear accumulators and counters
  float4 *accum = (float4 *)scratch;
  WfCounters *counters = (WfCounters *)((uint8_t *)scratch + kNoallocAccumBytes);
  TPT_CUDA(cudaMemsetAsync(accum, 0, npix * sizeof(float4), stream));
  TPT_CUDA(cudaMemsetAsync(counters, 0, sizeof(WfCounters), stream));
  const FrameDesc F{p->width, p->height, p->spp, npix * (unsigned long long)p->spp, accum, nullptr};
  const RenderCfg cfg{p->max_depth, p->semantics, p->background, p->sky_scale,
                      make_uint2((uint32_t)p->seed, (uint32_t)(p->seed >> 32)), p->refill > 0 ? p->refill : 1};
  const PersistentKernel kern = persistent_variant(p->wave, d.feat);
  const int smem = stack_smem(block);
  TPT_CUDA(smem_optin(kern, smem));
  int per_sm = 0;
  TPT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, block, smem));
  const int grid = sm_count * (per_sm < 1 ? 1 : per_sm);
  kern<<<grid, block, smem, stream>>>(d, cfg, F, counters);
  TPT_CUDA(cudaGetLastError());
  const int rgrid = (int)std::min<unsigned long long>((npix + 255) / 256, (unsigned long long)sm_count * 16);
  k_resolve<<<rgrid, 256, 0, stream>>>(F, out_rgb_dev);
  TPT_CUDA(cudaGetLastError());
  int err = 0;
  TPT_CUDA(cudaMemcpyAsync(&err, &counters->err, sizeof(int), cudaMemcpyDeviceToHost, stream));
  TPT_CUDA(cudaStreamSynchronize(stream));
  return err ? (tpt_status)err : TPT_OK;
}
