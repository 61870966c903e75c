// k_tc_gemm.cu -- BF16 GEMM on the fifth-generation tensor cores (tcgen05).
//
//   C[M][N] (fp32 or bf16, row stride ldc) = A[M][K] (bf16, K contiguous)
//                                            * B[N][K]^T (bf16, K contiguous)
//
// batched over blockIdx.z (B read at K offset z * b_kofs, C at z * c_batch),
// optionally banded: a CTA on rows [m0, m0 + 128) reduces only over
// K in [m0 - band, m0 + 128 + band) (rounded out to 64-element blocks), for
// banded (Toeplitz) A.
//
// One CTA computes a 128 x 128 tile of C.  Operands move global -> shared
// by TMA (cp.async.bulk.tensor, 128-byte swizzle, 64-element K blocks) in a
// kStages-deep ring guarded by mbarriers; one thread issues tcgen05.mma
// (kind::f16, BF16 x BF16 -> FP32) into a 128 x 128 FP32 accumulator in
// tensor memory; the four warps read the accumulator back with tcgen05.ld
// (warp w owns TMEM lanes = tile rows 32w .. 32w + 31) and store it.
//
// Every wait is bounded: after kSpinLimit polls the waiting thread sets bit 8
// of *err and gives up; the CTA still frees its tensor memory before it
// returns, so a failed launch leaves the device usable.
//
// Operand rows past M / N and K columns past K are read as zeros (TMA
// out-of-bounds fill); rows past M / N are not stored.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "pa_internal.cuh"
#include "tc_common.cuh"

namespace pa {
namespace {

constexpr int kBM = 128, kBN = 128, kBK = 64, kStages = 3;
constexpr int kTileBytesA = kBM * kBK * 2;  // 16 KB
constexpr int kTileBytesB = kBN * kBK * 2;  // 16 KB
constexpr int kStageBytes = kTileBytesA + kTileBytesB;
constexpr int kGemmThreads = 128;

using tc::mbar_arrive_expect_tx;
using tc::mbar_init;
using tc::mbar_wait;
using tc::smem_u32;
using tc::sw128_desc;
using tc::tma_load_2d;

// Instruction descriptor: D fp32, A and B bf16, both K-major, M = 128, N = 128.
constexpr uint32_t kIdesc = tc::idesc_bf16(kBM, kBN);

// Store 16 consecutive accumulator columns of one output row (fp32 or
// bf16; vector stores when the row segment is aligned and complete).
__device__ __forceinline__ void store16(const GemmArgs &g, int64_t cbase, int n,
                                        const uint32_t (&v)[16]) {
  const int N = g.N;
  if (g.out_bf16) {
    __nv_bfloat16 *crow = reinterpret_cast<__nv_bfloat16 *>(g.C) + cbase + n;
    if (n + 16 <= N && g.vec_ok) {
      uint32_t h[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const __nv_bfloat162 q =
            __floats2bfloat162_rn(__uint_as_float(v[2 * j]), __uint_as_float(v[2 * j + 1]));
        h[j] = *reinterpret_cast<const uint32_t *>(&q);
      }
      reinterpret_cast<uint4 *>(crow)[0] = make_uint4(h[0], h[1], h[2], h[3]);
      reinterpret_cast<uint4 *>(crow)[1] = make_uint4(h[4], h[5], h[6], h[7]);
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (n + j < N) crow[j] = __float2bfloat16_rn(__uint_as_float(v[j]));
    }
  } else {
    float *crow = reinterpret_cast<float *>(g.C) + cbase + n;
    if (n + 16 <= N && g.vec_ok) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        reinterpret_cast<float4 *>(crow)[j] =
            make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                        __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3]));
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (n + j < N) crow[j] = __uint_as_float(v[j]);
    }
  }
}

__global__ void __launch_bounds__(kGemmThreads, 2)
    k_tc_gemm_bf16(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   GemmArgs g, int *err) {
  const int M = g.M;
  extern __shared__ uint8_t smraw[];
  // tiles need 1024-byte alignment (swizzle atoms)
  uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accum;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN, z = blockIdx.z;
  int k_lo = 0, k_hi = g.K;
  if (g.band >= 0) {
    k_lo = max(0, m0 - g.band) & ~(kBK - 1);
    k_hi = min(g.K, m0 + kBM + g.band);
  }
  const int nk = k_hi > k_lo ? (k_hi - k_lo + kBK - 1) / kBK : 0;
  const int kb_ofs = z * g.b_kofs;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // 128 columns: the 128 x 128 fp32 accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(kBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStages;
      if (kb >= kStages && !mbar_wait(&empty[s], ((kb / kStages) - 1) & 1, err)) break;
      uint8_t *a = sm + s * kStageBytes;
      uint8_t *b = a + kTileBytesA;
      mbar_arrive_expect_tx(&full[s], kStageBytes);
      tma_load_2d(a, &tmA, k_lo + kb * kBK, m0, &full[s]);
      tma_load_2d(b, &tmB, kb_ofs + k_lo + kb * kBK, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % kStages;
      if (!mbar_wait(&full[s], (kb / kStages) & 1, err)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a = smem_u32(sm + s * kStageBytes);
      const uint32_t b = a + kTileBytesA;
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk) {  // K = 16 per instruction: +32 B
        const uint64_t da = sw128_desc(a + kk * 32);
        const uint64_t db = sw128_desc(b + kk * 32);
        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
            : "memory");
      }
      // the stage is free once these MMAs have read it
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&empty[s]))
          : "memory");
    }
    if (ok)
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&accum))
          : "memory");
  }
  __syncwarp();

  // epilogue: all four warps wait for the accumulator (an empty K range is
  // an all-zero tile and never touches it)
  bool ready = true;
  if (lane == 0 && nk > 0) ready = mbar_wait(&accum, 0, err);
  ready = __shfl_sync(0xFFFFFFFFu, ready ? 1 : 0, 0) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ready) {
    const int row = m0 + warp * 32 + lane;
    const int64_t cbase = (int64_t)z * g.c_batch + (int64_t)row * g.ldc;
#pragma unroll 1
    for (int c0 = 0; c0 < kBN; c0 += 16) {
      uint32_t v[16];
      if (nk == 0) {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0u;
      } else {
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
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
      if (row < M) store16(g, cbase, n0 + c0, v);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBN)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// Banded persistent variant (banded A, e.g. a Toeplitz filter matrix): a CTA
// keeps the band of A for its 128 rows resident in shared memory (at most
// kBandKB 64-wide K blocks), walks N tiles t = blockIdx.y, + gridDim.y, ...,
// streams their B blocks through a kBStages ring, and double-buffers the
// accumulator in tensor memory (2 x 128 columns) so that the epilogue of
// tile j runs while the MMAs of tile j + 1 are issued.  Warp 0: TMA
// producer; warp 1: MMA issuer; warps 2-5: epilogue (warp w reads TMEM lanes
// 32 (w % 4) .. 32 (w % 4) + 31).
// ---------------------------------------------------------------------------
constexpr int kBandKB = 6, kBStages = 4, kBandThreads = 192;
constexpr int kBandSmem = kBandKB * kTileBytesA + kBStages * kTileBytesB + 1024;

__global__ void __launch_bounds__(kBandThreads, 1)
    k_tc_gemm_band(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   GemmArgs g, int n_tiles_n, int *err) {
  extern __shared__ uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint8_t *sa = sm;                                // [kBandKB] A blocks
  uint8_t *sb = sm + kBandKB * kTileBytesA;        // [kBStages] B blocks
  __shared__ __align__(8) uint64_t a_full, bfull[kBStages], bempty[kBStages], acc_full[2],
      acc_empty[2];
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, z = blockIdx.z;
  const int k_lo = max(0, m0 - g.band) & ~(kBK - 1);
  const int k_hi = min(g.K, m0 + kBM + g.band);
  const int nk = k_hi > k_lo ? (k_hi - k_lo + kBK - 1) / kBK : 0;  // host: <= kBandKB
  const int kb_ofs = z * g.b_kofs;

  if (threadIdx.x == 0) {
    mbar_init(&a_full, 1);
    for (int s = 0; s < kBStages; ++s) {
      mbar_init(&bfull[s], 1);
      mbar_init(&bempty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&acc_full[a], 1);
      mbar_init(&acc_empty[a], 4);  // one arrive per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // two 128-column fp32 accumulators
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(2 * kBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (nk > 0 && warp == 0 && lane == 0) {
    // producer: the A band once, then the B blocks of every tile
    mbar_arrive_expect_tx(&a_full, nk * kTileBytesA);
    for (int kb = 0; kb < nk; ++kb) tma_load_2d(sa + kb * kTileBytesA, &tmA, k_lo + kb * kBK, m0, &a_full);
    int it = 0;
    bool ok = true;
    for (int t = blockIdx.y; t < n_tiles_n && ok; t += gridDim.y)
      for (int kb = 0; kb < nk; ++kb, ++it) {
        const int s = it % kBStages;
        if (it >= kBStages && !mbar_wait(&bempty[s], ((it / kBStages) - 1) & 1, err)) {
          ok = false;
          break;
        }
        mbar_arrive_expect_tx(&bfull[s], kTileBytesB);
        tma_load_2d(sb + s * kTileBytesB, &tmB, kb_ofs + k_lo + kb * kBK, t * kBN, &bfull[s]);
      }
  } else if (nk > 0 && warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = mbar_wait(&a_full, 0, err);
    int it = 0, j = 0;
    for (int t = blockIdx.y; t < n_tiles_n && ok; t += gridDim.y, ++j) {
      const int acc = j & 1;
      if (j >= 2 && !mbar_wait(&acc_empty[acc], ((j >> 1) - 1) & 1, err)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kb = 0; kb < nk; ++kb, ++it) {
        const int s = it % kBStages;
        if (!mbar_wait(&bfull[s], (it / kBStages) & 1, err)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a = smem_u32(sa + kb * kTileBytesA);
        const uint32_t b = smem_u32(sb + s * kTileBytesB);
#pragma unroll
        for (int kk = 0; kk < kBK / 16; ++kk) {
          const uint64_t da = sw128_desc(a + kk * 32);
          const uint64_t db = sw128_desc(b + kk * 32);
          const uint32_t accum_in = (kb > 0 || kk > 0) ? 1u : 0u;
          asm volatile(
              "{\n\t.reg .pred p;\n\t"
              "setp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                  tmem + (uint32_t)(acc * kBN)),
              "l"(da), "l"(db), "r"(kIdesc), "r"(accum_in)
              : "memory");
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&bempty[s]))
            : "memory");
      }
      if (!ok) break;
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&acc_full[acc]))
          : "memory");
    }
  } else if (warp >= 2) {
    // epilogue
    const int lg = warp & 3;  // TMEM lane group of this warp
    const int row = m0 + lg * 32 + lane;
    int j = 0;
    for (int t = blockIdx.y; t < n_tiles_n; t += gridDim.y, ++j) {
      const int acc = j & 1, n0 = t * kBN;
      bool ready = true;
      if (nk > 0) {
        if (lane == 0) ready = mbar_wait(&acc_full[acc], (j >> 1) & 1, err);
        ready = __shfl_sync(0xFFFFFFFFu, ready ? 1 : 0, 0) != 0;
        if (!ready) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      }
      const int64_t cbase = (int64_t)z * g.c_batch + (int64_t)row * g.ldc;
#pragma unroll 1
      for (int c0 = 0; c0 < kBN; c0 += 16) {
        uint32_t v[16];
        if (nk == 0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) v[q] = 0u;
        } else {
          const uint32_t taddr =
              tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(acc * kBN + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, "
              "%10, %11, %12, %13, %14, %15}, [%16];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
              : "r"(taddr)
              : "memory");
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        }
        if (row < g.M) store16(g, cbase, n0 + c0, v);
      }
      if (nk > 0) {
        // this warp's reads of the accumulator are complete
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0)
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[acc]))
                       : "memory");
      }
    }
  }
  __syncwarp();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kBN)
                 : "memory");
  }
}

bool make_map(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows, uint64_t row_bytes) {
  return tc::make_map_2d(m, base, cols, rows, row_bytes, kBK, kBM);
}

}  // namespace

cudaError_t launch_tc_gemm(const void *A, int64_t lda, int64_t a_rows, int64_t a_cols,
                           const void *B, int64_t ldb, int64_t b_rows, int64_t b_cols,
                           const GemmArgs &g0, int batch, int *err, cudaStream_t s) {
  GemmArgs g = g0;
  // TMA: 16-byte aligned bases and row strides (lda, ldb in elements); the
  // batch offset of B is a TMA coordinate and must be a multiple of 8
  if (g.M < 1 || g.N < 1 || g.K < 1 || batch < 1 || batch > 65535 || ((uintptr_t)A & 15) ||
      ((uintptr_t)B & 15) || (lda * 2) % 16 || (ldb * 2) % 16 || g.b_kofs % 8 || a_rows < g.M ||
      b_rows < g.N || g.ldc < g.N || a_cols > lda || b_cols > ldb || a_cols < 1 || b_cols < 1)
    return cudaErrorInvalidValue;
  const int esz = g.out_bf16 ? 2 : 4;
  g.vec_ok = ((uintptr_t)g.C % 16 == 0) && (g.ldc * esz) % 16 == 0 && (g.c_batch * esz) % 16 == 0;
  CUtensorMap ma, mb;
  if (!make_map(&ma, A, (uint64_t)a_cols, (uint64_t)a_rows, (uint64_t)lda * 2) ||
      !make_map(&mb, B, (uint64_t)b_cols, (uint64_t)b_rows, (uint64_t)ldb * 2))
    return cudaErrorInvalidValue;
  if (g.band >= 0) {
    // banded: the persistent kernel when every M tile's band fits its
    // resident A blocks
    int max_nk = 0;
    for (int m0 = 0; m0 < g.M; m0 += kBM) {
      const int lo = std::max(0, m0 - g.band) & ~(kBK - 1);
      const int hi = std::min(g.K, m0 + kBM + g.band);
      max_nk = std::max(max_nk, hi > lo ? (hi - lo + kBK - 1) / kBK : 0);
    }
    if (max_nk <= kBandKB) {
      cudaError_t e = cudaFuncSetAttribute(k_tc_gemm_band,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, kBandSmem);
      if (e != cudaSuccess) return e;
      int dev = 0, sms = 152;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      const int mt = (g.M + kBM - 1) / kBM, nt = (g.N + kBN - 1) / kBN;
      int gy = (int)std::max<int64_t>(1, (int64_t)sms / ((int64_t)mt * batch));
      gy = std::min(gy, nt);
      dim3 grid((unsigned)mt, (unsigned)gy, (unsigned)batch);
      k_tc_gemm_band<<<grid, kBandThreads, kBandSmem, s>>>(ma, mb, g, nt, err);
      return cudaGetLastError();
    }
  }
  const int smem = kStages * kStageBytes + 1024;
  cudaError_t e = cudaFuncSetAttribute(k_tc_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smem);
  if (e != cudaSuccess) return e;
  dim3 grid((unsigned)((g.M + kBM - 1) / kBM), (unsigned)((g.N + kBN - 1) / kBN), (unsigned)batch);
  k_tc_gemm_bf16<<<grid, kGemmThreads, smem, s>>>(ma, mb, g, err);
  return cudaGetLastError();
}

cudaError_t launch_tc_gemm_bf16(const void *A, int64_t lda, const void *B, int64_t ldb, float *C,
                                int64_t ldc, int M, int N, int K, int *err, cudaStream_t s) {
  if (lda < K || ldb < K) return cudaErrorInvalidValue;
  GemmArgs g{};
  g.C = C;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ldc = ldc;
  g.band = -1;
  return launch_tc_gemm(A, lda, M, K, B, ldb, N, K, g, 1, err, s);
}

namespace tc {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

bool make_map_2d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows,
                 uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {row_bytes};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_map_f32_2d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows,
                     uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {row_bytes};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_map_f32_3d(CUtensorMap *m, const void *base, uint64_t cols, uint64_t rows,
                     uint64_t planes, uint32_t box_cols, uint32_t box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[3] = {cols, rows, planes};
  const cuuint64_t strides[2] = {cols * 4, cols * 4 * rows};
  const cuuint32_t box[3] = {box_cols, box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_map_nhwc(CUtensorMap *m, const void *base, uint64_t C, uint64_t W, uint64_t H,
                   uint64_t N, uint32_t box_w) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[4] = {C, W, H, N};
  const cuuint64_t strides[3] = {C * 2, C * 2 * W, C * 2 * W * H};
  const cuuint32_t box[4] = {64, box_w, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims, strides, box,
             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc
}  // namespace pa
