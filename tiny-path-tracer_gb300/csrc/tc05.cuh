// tc05.cuh - Blackwell (sm_103a) tensor-core building blocks in inline PTX:
// tcgen05.mma (kind::f16, f32 accumulators in tensor memory), tensor-memory
// allocation and loads, mbarrier waits with a time limit, and the shared-
// memory operand layout the MMAs read.
//
// Operand layout: 128-byte swizzled tiles of 64 f16 columns.  Row r of a
// tile occupies bytes [128 r, 128 r + 128); its 16-byte chunk c (columns
// 8c..8c+7) sits at chunk position c ^ (r mod 8).  Tiles start on a 1024-byte
// boundary (one swizzle atom = 8 rows).  The same bytes serve as a K-major
// operand (rows = M or N, columns = K) and, read through an MN-major
// descriptor, as the transposed operand (columns = M or N, rows = K), which
// is how the backward pass and the weight gradients reuse the forward
// tiles without transposed copies.
//
// Descriptors (64-bit shared-memory matrix descriptor of tcgen05): start
// address >> 4 in bits 0-13, leading-dimension byte offset >> 4 in bits
// 16-29, stride-dimension byte offset >> 4 in bits 32-45, descriptor version
// 1 in bits 46-47, swizzle mode in bits 61-63 (2 = 128-byte).  K-major
// swizzled tiles: stride = 1024 bytes between 8-row groups, a K step of 16
// elements advances the start address by 32 bytes inside the atom.
// MN-major: stride = 1024 bytes between 8-row (K) groups, leading offset =
// bytes between 64-column blocks, a K step of 16 rows advances the start by
// 2048 bytes.  The 32-bit instruction descriptor: accumulator format in bits
// 4-5 (1 = f32), A / B formats in bits 7-9 / 10-12 (0 = f16), A / B major in
// bits 15 / 16 (1 = MN-major), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
//
// Accumulator layouts in tensor memory (checked on a GB300): M = 128, row i
// in lane i; M = 64, rows 16w..16w+15 in lanes 32w..32w+15 (warp w's
// quarter, its first 16 lanes).  Columns are the N index.
#ifndef TPT_TC05_CUH
#define TPT_TC05_CUH

#include <cuda_fp16.h>
#include <stdint.h>

namespace tpt {
namespace tc05 {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, col) in a swizzled tile of 64 f16 columns
__host__ __device__ __forceinline__ uint32_t sw128(int row, int col) {
  return (uint32_t)(row * 128 + ((((col >> 3) ^ (row & 7)) & 7) << 4) + (col & 7) * 2);
}
// byte offset of 16-byte chunk c (columns 8c..8c+7) of row `row`
__host__ __device__ __forceinline__ uint32_t sw128_chunk(int row, int c) {
  return (uint32_t)(row * 128 + (((c ^ (row & 7)) & 7) << 4));
}

__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32) | (1ull << 46) | (2ull << 61);
}

__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, bool a_mn, bool b_mn) {
  return (1u << 4) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// D (tensor memory) = A * B (+ D if accumulate); issued by one thread
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}
// the mbarrier's phase completes when every MMA this thread issued so far is done
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Waits for the phase with the given parity; gives up after `limit` clock
// cycles (returns false) so a lost arrival cannot hang the kernel.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > limit) return false;
  }
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the MMAs (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16-byte global -> shared copy in the background; src_bytes = 0 zero-fills
__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(dst_smem)), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Bulk copy global -> shared (16-byte aligned, size a multiple of 16) that
// completes on an mbarrier; the issuing thread first announces the bytes the
// phase waits for (arrive + expect_tx, one arrival).
__device__ __forceinline__ void bar_expect_bytes(uint32_t bar, uint32_t bytes) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(bar),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy(uint32_t dst_smem, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst_smem),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// a descriptor for the operand `bytes` further on (addresses stay below 256 KB)
__device__ __forceinline__ uint64_t desc_add(uint64_t d, uint32_t bytes) { return d + (uint64_t)(bytes >> 4); }

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while its predecessor in the stream still runs;
// griddep_wait blocks the calling thread until the predecessor grids have
// completed and their memory is visible, griddep_launch lets this grid's
// own dependents start (once every CTA has issued it or exited).  Without
// the launch attribute both return at once.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// gradient[addr..addr+3] += v without a return value (16-byte aligned)
__device__ __forceinline__ void red_add_v4(float *addr, float4 v) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
}

// one warp: allocate / free `ncols` tensor-memory columns (power of two >= 32)
__device__ __forceinline__ void tmem_alloc(uint32_t *slot_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 64 consecutive 32-bit columns of this thread's lane (32x32b shape): warp w
// reads lanes 32w..32w+31 of the address's lane field + the column offset.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
      "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
      "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 64; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc05
}  // namespace tpt
#endif
