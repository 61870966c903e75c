// tc_common.cuh -- primitives shared by the tcgen05 kernels: mbarriers with
// bounded waits, TMA tile loads, shared-memory matrix descriptors for
// 128-byte-swizzled tiles and the tensor-map encoder.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pa {
namespace tc {

constexpr uint32_t kSpinLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Ends the barrier's life (no thread may still wait on it); the memory can
// then hold a new barrier.
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Non-blocking probe of phase `parity`; the caller bounds the polling.
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Blocking probe: the thread may be suspended until the phase completes or
// a hardware time limit passes; the caller bounds the retries.
__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits with mbar_try, at most kTryLimit retries; on time-out sets bit 8 of
// *err.
constexpr uint32_t kTryLimit = 1u << 20;
__device__ __forceinline__ bool mbar_wait_try(uint64_t *bar, uint32_t parity, int *err) {
  for (uint32_t i = 0; i < kTryLimit; ++i)
    if (mbar_try(bar, parity)) return true;
  atomicOr(err, 8);
  return false;
}

// Polls at most kSpinLimit times; on time-out sets bit 8 of *err.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
  for (uint32_t i = 0; i < kSpinLimit; ++i)
    if (mbar_test(bar, parity)) return true;
  atomicOr(err, 8);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Untiled bulk copy global -> shared (both 16-byte aligned, bytes a
// multiple of 16), completing on `bar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Starts bringing [src, src + bytes) into L2 (16-byte aligned, bytes a
// multiple of 16).
__device__ __forceinline__ void bulk_prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c, int x, int y,
                                            int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of an operand tile stored as TMA writes
// it with 128-byte swizzle (rows of 128 B, 8-row atoms of 1024 B, tile base
// 1024-byte aligned).  K-major tiles: `lbo` is unused and `sbo` (1024) steps
// between 8-row groups along M / N.  MN-major tiles (rows run along K): `lbo`
// steps between 64-element atoms along M / N and `sbo` (1024) between 8-row
// groups along K.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr, uint32_t lbo = 16,
                                               uint32_t sbo = 1024) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);      // start address
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;   // leading byte offset
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;                        // descriptor version
  d |= (uint64_t)2 << 61;                        // 128-byte swizzle
  return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D fp32, A and B bf16,
// M x N tile; `a_mn` / `b_mn` select MN-major (transposed) operands.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn = false,
                                                  bool b_mn = false) {
  return (1u << 4)                     // D format: f32
         | (1u << 7)                   // A format: bf16
         | (1u << 10)                  // B format: bf16
         | ((a_mn ? 1u : 0u) << 15)    // A major-ness
         | ((b_mn ? 1u : 0u) << 16)    // B major-ness
         | ((uint32_t)(N >> 3) << 17)  //
         | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives on `bar` once every tcgen05.mma issued so far by this thread has
// completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive fp32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t tmem, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols)
               : "memory");
}

// Host: bf16 tensor maps with 128-byte swizzle and zero fill outside the
// tensor.  2-D: `rows` rows of `cols` elements (row stride in bytes), box
// box_cols x box_rows.  4-D (NHWC activations): dims {C, W, H, N}, box
// {64, box_w, 1, 1}.
bool make_map_2d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows,
                 uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows);
bool make_map_nhwc(CUtensorMap *m, const void *base, uint64_t C, uint64_t W, uint64_t H,
                   uint64_t N, uint32_t box_w);
// fp32 2-D map without swizzle, zero fill outside: `rows` rows of `cols`
// floats (row stride in bytes, a multiple of 16), box box_cols x box_rows.
bool make_map_f32_2d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows,
                     uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows);
// fp32 3-D map of a dense [planes][rows][cols] array, box box_cols x box_rows
// x 1, zero fill outside every dimension.
bool make_map_f32_3d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows,
                     uint64_t planes, uint32_t box_cols, uint32_t box_rows);

}  // namespace tc
}  // namespace pa
