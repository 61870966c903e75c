// k_conv.cu -- the learned unary's convolutions on the tcgen05 tensor cores.
//
// Activations are NHWC bf16: [field][row][column][channel], 64 channels per
// hidden layer, `dim` (a multiple of 64) for the descriptor field.  Weights
// are [out channel][tap][in channel] (taps 1 or 9, row-major over (dy, dx)).
//
// k_conv_igemm: implicit-GEMM convolution, forward or input gradient.  One
// CTA computes one row segment of 128 output positions x 64 output channels:
// for every tap (dy, dx) and 64-channel block it loads, by 4-D TMA, the 128
// input positions (x0 + dx .. x0 + dx + 127) of row y + dy -- positions
// outside the field arrive as zeros, which is the convolution's zero
// padding -- and the matching 64 x 64 weight block, and one thread issues
// tcgen05.mma (BF16 x BF16 -> FP32 in tensor memory).  The epilogue adds
// the bias and applies ReLU (hidden layers), writes FP32 scores (output
// layer, optionally exponentiated), or multiplies an input gradient by the
// ReLU mask of the layer below (backward).
//
// k_conv_wgrad: weight gradient dW[co][tap][ci] = sum over positions of
// dZ[pos][co] * X[pos + tap][ci].  The reduction runs over positions, which
// are the rows of both NHWC tensors, so both operands enter the MMA
// MN-major straight from their TMA tiles (64 positions x 64 channels): the
// accumulator is 128 (two tap/channel-block atoms) x 64 (co).  Positions are
// split over CTAs; each CTA writes its partial sums and k_wgrad_reduce adds
// them in a fixed order (deterministic results).
//
// k_conv3_persist: the 3x3, 64-channel layers as persistent CTAs (resident
// weights, each input row loaded once per output row segment, double-buffered
// accumulators; see below).  k_conv_igemm serves the 1x1 layer: one row
// segment per CTA, two CTAs per SM, measured faster there than a persistent
// form whose resident weights leave room for fewer loads in flight.
//
// Every mbarrier wait is bounded (bit 8 of *err on time-out) and tensor
// memory is freed on every path.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "pa_internal.cuh"
#include "tc_common.cuh"

namespace pa {
namespace {

using tc::mbar_arrive_expect_tx;
using tc::mbar_init;
using tc::mbar_wait;
using tc::smem_u32;
using tc::sw128_desc;

constexpr int kCM = 128;  // output positions per CTA tile
constexpr int kCN = 64;   // output channels per CTA tile
constexpr int kCK = 64;   // channels per K block
constexpr int kStagesC = 4;
constexpr int kABytes = kCM * kCK * 2;  // 16 KB
constexpr int kBBytes = kCN * kCK * 2;  // 8 KB
constexpr int kStageC = kABytes + kBBytes;
constexpr int kConvSmem = kStagesC * kStageC + 1024;
constexpr int kConvThreads = 128;
constexpr uint32_t kIdescConv = tc::idesc_bf16(kCM, kCN);

// weight gradient: two 64-row atoms of X and one of dZ per stage
constexpr int kWAtom = 64 * kCK * 2;  // 8 KB
constexpr int kWStage = 3 * kWAtom;
constexpr int kWSmem = kStagesC * kWStage + 1024;
constexpr uint32_t kIdescWgrad = tc::idesc_bf16(128, kCN, true, true);

__device__ __forceinline__ void tap_shift(int taps, int t, int &dy, int &dx) {
  if (taps == 9) {
    dy = t / 3 - 1;
    dx = t % 3 - 1;
  } else {
    dy = 0;
    dx = 0;
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 q = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&q);
}

// Epilogue of one thread's output position: 16 accumulator columns from
// c0, stored as the layer's mode asks (ConvArgs).
__device__ __forceinline__ void conv_store16(const ConvArgs &a, int64_t pos, int f, int y, int x,
                                             int c0, const uint32_t (&v)[16]) {
  if (a.mode == kConvReluBf16) {
    uint32_t h[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      h[j] = pack_bf16(fmaxf(__uint_as_float(v[2 * j]) + a.bias[c0 + 2 * j], 0.f),
                       fmaxf(__uint_as_float(v[2 * j + 1]) + a.bias[c0 + 2 * j + 1], 0.f));
    uint4 *o = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(a.out) + pos * kCN + c0);
    o[0] = make_uint4(h[0], h[1], h[2], h[3]);
    o[1] = make_uint4(h[4], h[5], h[6], h[7]);
  } else if (a.mode == kConvMaskBf16) {
    const uint4 *m = reinterpret_cast<const uint4 *>(a.act + pos * kCN + c0);
    const uint4 m0 = m[0], m1 = m[1];
    const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
    uint32_t h[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const __nv_bfloat162 q = *reinterpret_cast<const __nv_bfloat162 *>(&mw[j]);
      const float lo = __low2float(q) > 0.f ? __uint_as_float(v[2 * j]) : 0.f;
      const float hi = __high2float(q) > 0.f ? __uint_as_float(v[2 * j + 1]) : 0.f;
      h[j] = pack_bf16(lo, hi);
    }
    uint4 *o = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(a.out) + pos * kCN + c0);
    o[0] = make_uint4(h[0], h[1], h[2], h[3]);
    o[1] = make_uint4(h[4], h[5], h[6], h[7]);
  } else {
    float *o = reinterpret_cast<float *>(a.out) + (int64_t)f * a.out_sf + (int64_t)y * a.W + x;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int c = c0 + j;
      if (c < a.n_out) {
        float val = __uint_as_float(v[j]) + a.bias[c];
        if (a.exp_out) val = expf(val);
        o[(int64_t)c * a.out_sc] = val;
      }
    }
  }
}

__global__ void __launch_bounds__(kConvThreads, 2)
    k_conv_igemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 ConvArgs a, int *err) {
  extern __shared__ uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStagesC], empty[kStagesC], accum;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // a.flat (1x1 layers): the tile is 128 consecutive positions of the
  // flattened [field][row][column] index, read through a 2-D map
  const int x0 = blockIdx.x * kCM, y = blockIdx.y, f = blockIdx.z;
  const int64_t p0 = (int64_t)blockIdx.x * kCM;
  const int nk = a.taps * a.cin_blocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStagesC; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kCN);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {
    // TMA producer: K block kb = (tap, channel block)
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStagesC;
      if (kb >= kStagesC && !mbar_wait(&empty[s], ((kb / kStagesC) - 1) & 1, err)) break;
      const int t = kb / a.cin_blocks, cb = kb - t * a.cin_blocks;
      int dy, dx;
      tap_shift(a.taps, t, dy, dx);
      uint8_t *sa = sm + s * kStageC;
      mbar_arrive_expect_tx(&full[s], kStageC);
      if (a.flat) tc::tma_load_2d(sa, &tmA, cb * kCK, (int)p0, &full[s]);
      else tc::tma_load_4d(sa, &tmA, cb * kCK, x0 + dx, y + dy, f, &full[s]);
      tc::tma_load_2d(sa + kABytes, &tmB, kb * kCK, 0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % kStagesC;
      if (!mbar_wait(&full[s], (kb / kStagesC) & 1, err)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = smem_u32(sm + s * kStageC);
      const uint32_t sb = sa + kABytes;
#pragma unroll
      for (int kk = 0; kk < kCK / 16; ++kk)  // K = 16 per instruction: +32 B
        tc::mma_bf16(tmem, sw128_desc(sa + kk * 32), sw128_desc(sb + kk * 32), kIdescConv,
                     (kb > 0 || kk > 0) ? 1u : 0u);
      tc::mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
    }
    if (ok) tc::mma_commit(&accum);
  }
  __syncwarp();

  bool ready = true;
  if (lane == 0) ready = mbar_wait(&accum, 0, err);
  ready = __shfl_sync(0xFFFFFFFFu, ready ? 1 : 0, 0) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ready) {
    int64_t pos;
    int pf = f, py = y, px = x0 + warp * 32 + lane;
    bool live;
    if (a.flat) {
      pos = p0 + warp * 32 + lane;
      const int64_t hw = (int64_t)a.H * a.W;
      live = pos < (int64_t)a.n * hw;
      pf = (int)(pos / hw);
      const int yx = (int)(pos - pf * hw);
      py = yx / a.W;
      px = yx - py * a.W;
    } else {
      live = px < a.W;
      pos = ((int64_t)f * a.H + y) * a.W + px;
    }
    const int c_end = a.mode == kConvOutF32 ? a.n_out : kCN;
#pragma unroll 1
    for (int c0 = 0; c0 < c_end; c0 += 16) {
      uint32_t v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (live) conv_store16(a, pos, pf, py, px, c0, v);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tc::tmem_dealloc(tmem, kCN);
  }
}

__global__ void __launch_bounds__(kConvThreads, 2)
    k_conv_wgrad(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmD,
                 WgradArgs w, int *err) {
  extern __shared__ uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  __shared__ __align__(8) uint64_t full[kStagesC], empty[kStagesC], accum;
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x, split = blockIdx.y;
  const int k_lo = split * w.kb_per_split;
  const int k_hi = min(w.kblocks, k_lo + w.kb_per_split);
  const int nk = max(0, k_hi - k_lo);
  // the two atoms (tap, channel block) of this tile; an odd last tile
  // repeats its first atom and does not store the second
  const int a0 = 2 * mt, a1 = (2 * mt + 1 < w.n_atoms) ? 2 * mt + 1 : 2 * mt;
  const int t0 = a0 / w.cin_blocks, cb0 = a0 - t0 * w.cin_blocks;
  const int t1 = a1 / w.cin_blocks, cb1 = a1 - t1 * w.cin_blocks;
  int dy0, dx0, dy1, dx1;
  tap_shift(w.taps, t0, dy0, dx0);
  tap_shift(w.taps, t1, dy1, dx1);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStagesC; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, kCN);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {
    for (int i = 0; i < nk; ++i) {
      const int s = i % kStagesC;
      if (i >= kStagesC && !mbar_wait(&empty[s], ((i / kStagesC) - 1) & 1, err)) break;
      const int kb = k_lo + i;
      const int xi = kb % w.xb, r = kb / w.xb;
      const int y = r % w.H, f = r / w.H, x0 = xi * 64;
      uint8_t *st = sm + s * kWStage;
      mbar_arrive_expect_tx(&full[s], kWStage);
      tc::tma_load_4d(st, &tmX, cb0 * kCK, x0 + dx0, y + dy0, f, &full[s]);
      tc::tma_load_4d(st + kWAtom, &tmX, cb1 * kCK, x0 + dx1, y + dy1, f, &full[s]);
      tc::tma_load_4d(st + 2 * kWAtom, &tmD, 0, x0, y, f, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    bool ok = true;
    for (int i = 0; i < nk; ++i) {
      const int s = i % kStagesC;
      if (!mbar_wait(&full[s], (i / kStagesC) & 1, err)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sx = smem_u32(sm + s * kWStage);
      const uint32_t sd = sx + 2 * kWAtom;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)  // K = 16 positions per instruction: +2048 B
        tc::mma_bf16(tmem, sw128_desc(sx + kk * 2048, kWAtom, 1024),
                     sw128_desc(sd + kk * 2048, kWAtom, 1024), kIdescWgrad,
                     (i > 0 || kk > 0) ? 1u : 0u);
      tc::mma_commit(&empty[s]);
    }
    if (ok && nk > 0) tc::mma_commit(&accum);
  }
  __syncwarp();

  bool ready = true;
  if (lane == 0 && nk > 0) ready = mbar_wait(&accum, 0, err);
  ready = __shfl_sync(0xFFFFFFFFu, ready ? 1 : 0, 0) != 0;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ready) {
    const int row = warp * 32 + lane;
    float4 *o = reinterpret_cast<float4 *>(w.part + (((int64_t)split * w.m_tiles + mt) * 128 + row) * kCN);
#pragma unroll 1
    for (int c0 = 0; c0 < kCN; c0 += 16) {
      uint32_t v[16];
      if (nk > 0) {
        tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0u;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        o[c0 / 4 + j] = make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                                    __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tc::tmem_dealloc(tmem, kCN);
  }
}

// ---------------------------------------------------------------------------
// k_conv3_persist: the 3x3, 64-channel layers (forward and input gradient).
// Persistent: one CTA per SM walks row segments t = blockIdx.x, +gridDim.x.
// The layer's nine 64 x 64 weight blocks stay resident in shared memory; per
// row segment the three input rows y-1, y, y+1 are loaded once (130
// positions x0-1 .. x0+128 each, zero-filled outside the field) and tap
// (dy, dx) reads rows dx+1 .. dx+128 of row tile dy+1: its A descriptor
// starts (dx+1) * 128 bytes into the tile.  Row tiles and accumulators are
// double-buffered: warp 0 loads tile j+1 and warp 1 issues its MMAs while
// warps 2..5 drain tile j from tensor memory.
// ---------------------------------------------------------------------------
constexpr int kRowPos = kCM + 2;                          // 130 positions per input row
constexpr int kRowTile = ((kRowPos * 128 + 1023) / 1024) * 1024;  // 17 KB
constexpr int kP3Threads = 192;
constexpr int kP3W = 9 * kBBytes;                         // resident weights, 72 KB
constexpr int kP3Smem = kP3W + 2 * 3 * kRowTile + 1024;

__global__ void __launch_bounds__(kP3Threads, 1)
    k_conv3_persist(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    ConvArgs a, int n_tiles, int *err) {
  extern __shared__ uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint8_t *sw = sm;                // [9] weight blocks (8 KB each)
  uint8_t *srow = sm + kP3W;       // [2][3] row tiles
  __shared__ __align__(8) uint64_t wfull, full[2], empty[2], acc_full[2], acc_empty[2];
  __shared__ uint32_t tmem_base;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int xt = (a.W + kCM - 1) / kCM;
  if (threadIdx.x == 0) {
    mbar_init(&wfull, 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], 1);
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);  // one arrive per epilogue warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, 2 * kCN);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0 && lane == 0) {
    mbar_arrive_expect_tx(&wfull, kP3W);
    for (int t = 0; t < 9; ++t) tc::tma_load_2d(sw + t * kBBytes, &tmB, t * kCK, 0, &wfull);
    int j = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++j) {
      const int b = j & 1;
      if (j >= 2 && !mbar_wait(&empty[b], ((j >> 1) - 1) & 1, err)) break;
      const int xi = tile % xt, r = tile / xt, y = r % a.H, f = r / a.H;
      mbar_arrive_expect_tx(&full[b], 3 * kRowPos * 128);
      for (int dy = 0; dy < 3; ++dy)
        tc::tma_load_4d(srow + (b * 3 + dy) * kRowTile, &tmA, 0, xi * kCM - 1, y + dy - 1, f,
                        &full[b]);
    }
  } else if (warp == 1 && lane == 0) {
    bool ok = mbar_wait(&wfull, 0, err);
    int j = 0;
    for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x, ++j) {
      const int b = j & 1;
      if (j >= 2 && !mbar_wait(&acc_empty[b], ((j >> 1) - 1) & 1, err)) break;
      if (!mbar_wait(&full[b], (j >> 1) & 1, err)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = tmem + (uint32_t)(b * kCN);
      for (int t = 0; t < 9; ++t) {
        const uint32_t sa = smem_u32(srow + (b * 3 + t / 3) * kRowTile) + (uint32_t)((t % 3) * 128);
        const uint32_t sb = smem_u32(sw + t * kBBytes);
#pragma unroll
        for (int kk = 0; kk < kCK / 16; ++kk)
          tc::mma_bf16(acc, sw128_desc(sa + kk * 32), sw128_desc(sb + kk * 32), kIdescConv,
                       (t > 0 || kk > 0) ? 1u : 0u);
      }
      tc::mma_commit(&empty[b]);     // the row tiles are free once read
      tc::mma_commit(&acc_full[b]);  // the accumulator is complete
    }
  } else if (warp >= 2) {
    const int lg = warp & 3;  // TMEM lane group of this warp
    int j = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++j) {
      const int b = j & 1;
      bool ready = true;
      if (lane == 0) ready = mbar_wait(&acc_full[b], (j >> 1) & 1, err);
      ready = __shfl_sync(0xFFFFFFFFu, ready ? 1 : 0, 0) != 0;
      if (!ready) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int xi = tile % xt, r = tile / xt, y = r % a.H, f = r / a.H;
      const int x = xi * kCM + lg * 32 + lane;
      const bool live = x < a.W;
      const int64_t pos = ((int64_t)f * a.H + y) * a.W + x;
      const int c_end = a.mode == kConvOutF32 ? a.n_out : kCN;
#pragma unroll 1
      for (int c0 = 0; c0 < c_end; c0 += 16) {
        uint32_t v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * kCN + c0), v);
        if (live) conv_store16(a, pos, f, y, x, c0, v);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[b]))
                     : "memory");
    }
  }
  __syncwarp();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tc::tmem_dealloc(tmem, 2 * kCN);
  }
}

// grad[co][t][ci] = sum over splits (in order) of the partial sums.
__global__ void k_wgrad_reduce(const float *__restrict__ part, int splits, int m_tiles,
                               int cin_blocks, int taps, int cout, float *__restrict__ grad) {
  const int cin = cin_blocks * 64;
  const int64_t total = (int64_t)cout * taps * cin;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int co = (int)(i / ((int64_t)taps * cin));
    const int rem = (int)(i - (int64_t)co * taps * cin);
    const int t = rem / cin, ci = rem - t * cin;
    const int at = t * cin_blocks + ci / 64;
    const int row = (at >> 1) * 128 + (at & 1) * 64 + (ci & 63);
    float acc = 0.f;
    for (int s = 0; s < splits; ++s) acc += part[(((int64_t)s * m_tiles) * 128 + row) * 64 + co];
    grad[i] = acc;
  }
}

// Bias gradient, pass 1: block b sums positions [b*chunk, (b+1)*chunk) of
// dZ [pos][64] per channel (4 rows of 64 threads, then in order).
__global__ void __launch_bounds__(256) k_bias_partial(const __nv_bfloat16 *__restrict__ dz,
                                                      int64_t n_pos, int64_t chunk,
                                                      float *__restrict__ part) {
  __shared__ float acc4[4][64];
  const int c = threadIdx.x & 63, r = threadIdx.x >> 6;
  const int64_t lo = blockIdx.x * chunk, hi = min(n_pos, lo + chunk);
  float acc = 0.f;
  for (int64_t p = lo + r; p < hi; p += 4) acc += __bfloat162float(dz[p * 64 + c]);
  acc4[r][c] = acc;
  __syncthreads();
  if (r == 0) part[(int64_t)blockIdx.x * 64 + c] = ((acc4[0][c] + acc4[1][c]) + acc4[2][c]) + acc4[3][c];
}

__global__ void k_bias_final(const float *__restrict__ part, int nb, int cout,
                             float *__restrict__ grad) {
  const int c = threadIdx.x;
  if (c >= cout) return;
  float acc = 0.f;
  for (int b = 0; b < nb; ++b) acc += part[(int64_t)b * 64 + c];
  grad[c] = acc;
}

// Squared error of the output layer against the reference's log scores of
// the AdaBoost maps (clip_scores_fill then log: s < 0 -> log 1e-4, s == 0
// is LOG_ZERO and left out of the loss), and its gradient dZ [pos][64]
// (channels >= P zero).  One thread per position; per-block loss sums.
__global__ void __launch_bounds__(256) k_loss_grad(LossArgs l, __nv_bfloat16 *__restrict__ dz,
                                                   float *__restrict__ loss_part) {
  __shared__ float red[256];
  const int64_t n_pos = (int64_t)l.n * l.H * l.W;
  const int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float loss = 0.f;
  if (pos < n_pos) {
    const int64_t hw = (int64_t)l.H * l.W;
    const int f = (int)(pos / hw);
    const int64_t yx = pos - (int64_t)f * hw;
    uint32_t h[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) h[j] = 0u;
    float g[2];
    for (int c = 0; c < l.P; ++c) {
      const float yv = l.pred[(int64_t)f * l.pred_sf + (int64_t)c * l.pred_sc + yx];
      const float s = l.scores[(int64_t)f * l.score_sf + (int64_t)c * l.score_sc + yx];
      float gv = 0.f;
      if (s != 0.f) {
        const float tgt = s < 0.f ? logf(1e-4f) : logf(s);
        const float d = yv - tgt;
        loss += d * d;
        gv = 2.f * d * l.inv_count;
      }
      g[c & 1] = gv;
      if (c & 1) h[c >> 1] = pack_bf16(g[0], g[1]);
      else if (c == l.P - 1) h[c >> 1] = pack_bf16(g[0], 0.f);
    }
    uint4 *o = reinterpret_cast<uint4 *>(dz + pos * 64);
#pragma unroll
    for (int j = 0; j < 8; ++j) o[j] = make_uint4(h[4 * j], h[4 * j + 1], h[4 * j + 2], h[4 * j + 3]);
  }
  red[threadIdx.x] = loss;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

__global__ void k_sum_final(const float *__restrict__ part, int n, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc += (double)part[i];
    *out = acc;
  }
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, int64_t n, AdamArgs a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = a.b1 * m[i] + (1.f - a.b1) * gi;
    const float vi = a.b2 * v[i] + (1.f - a.b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= a.lr * (mi / a.bc1) / (sqrtf(vi / a.bc2) + a.eps);
  }
}

// Master weights (fp32) -> the bf16 operands: forward [64][taps*cin] with
// rows >= cout zero, and for the 3x3 layers the input-gradient operand
// [ci][tap'][co] = W[co][8 - tap'][ci] (flipped taps, co padded to 64).
__global__ void k_pack_weights(const float *__restrict__ params, PackArgs a) {
  const int64_t n0 = (int64_t)64 * a.dim;
  const int64_t n3 = (int64_t)64 * 576;
  const int64_t total = n0 + 8 * n3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < n0) {
      a.wf0[i] = __float2bfloat16_rn(params[a.off_w[0] + i]);
      continue;
    }
    const int64_t j = i - n0;
    const int which = (int)(j / n3), l = 1 + (which & 3);
    const int e = (int)(j - (int64_t)which * n3);
    const int cout = l == 4 ? a.P : 64;
    const float *w = params + a.off_w[l];
    if (which < 4) {  // forward operand [co][k]
      const int co = e / 576, k = e - co * 576;
      a.wf[l - 1][e] = __float2bfloat16_rn(co < cout ? w[(int64_t)co * 576 + k] : 0.f);
    } else {  // input-gradient operand [ci][tap'][co]
      const int ci = e / 576, k = e - ci * 576, tp = k / 64, co = k - tp * 64;
      a.wd[l - 1][e] =
          __float2bfloat16_rn(co < cout ? w[((int64_t)co * 9 + (8 - tp)) * 64 + ci] : 0.f);
    }
  }
}

__global__ void k_cast_bf16(const float4 *__restrict__ src, uint2 *__restrict__ dst, int64_t n4) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = src[i];
    dst[i] = make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
  }
}

int grid_for(int64_t n, int threads) {
  return (int)std::min<int64_t>((n + threads - 1) / threads, 152 * 16);
}

int wgrad_splits(int m_tiles, int kblocks, int *kb_per_split) {
  int sms = 152, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int splits = std::max(1, std::min(kblocks, (2 * sms + m_tiles - 1) / m_tiles));
  const int per = (kblocks + splits - 1) / splits;
  *kb_per_split = per;
  return (kblocks + per - 1) / per;
}

}  // namespace

cudaError_t launch_conv(const void *in, int cin, int taps, int n, int H, int W, const void *wts,
                        const ConvArgs &a0, int *err, cudaStream_t s) {
  if (cin < 64 || cin % 64 || (taps != 1 && taps != 9) || n < 1 || n > 65535 || H < 1 ||
      H > 65535 || W < 1 || ((uintptr_t)in & 15) || ((uintptr_t)wts & 15) || !a0.out ||
      (a0.mode == kConvMaskBf16 && !a0.act) || (a0.mode != kConvMaskBf16 && !a0.bias) ||
      (a0.mode == kConvOutF32 && (a0.n_out < 1 || a0.n_out > 64)))
    return cudaErrorInvalidValue;
  ConvArgs a = a0;
  a.n = n;
  a.H = H;
  a.W = W;
  a.cin_blocks = cin / 64;
  a.taps = taps;
  CUtensorMap ma, mb;
  if (!tc::make_map_2d(&mb, wts, (uint64_t)taps * cin, 64, (uint64_t)taps * cin * 2, kCK, kCN))
    return cudaErrorInvalidValue;
  cudaError_t e;
  if (taps == 9 && cin == 64) {
    // 3x3 layers: persistent CTAs with resident weights and reused input rows
    if (!tc::make_map_nhwc(&ma, in, cin, W, H, n, kRowPos)) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(k_conv3_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, kP3Smem);
    if (e != cudaSuccess) return e;
    const int64_t n_tiles = (int64_t)n * H * ((W + kCM - 1) / kCM);
    if (n_tiles > 0x7FFFFFFF) return cudaErrorInvalidValue;
    int sms = 152, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<int64_t>(n_tiles, sms);
    k_conv3_persist<<<grid, kP3Threads, kP3Smem, s>>>(ma, mb, a, (int)n_tiles, err);
    return cudaGetLastError();
  }
  // 1x1: one GEMM over the flattened positions (full 128-position tiles)
  const int64_t n_pos = (int64_t)n * H * W;
  a.flat = taps == 1 && (n_pos + kCM - 1) / kCM <= 0x7FFFFFFF && n_pos <= 0x7FFFFFFF;
  if (a.flat ? !tc::make_map_2d(&ma, in, (uint64_t)cin, (uint64_t)n_pos, (uint64_t)cin * 2, kCK, kCM)
             : !tc::make_map_nhwc(&ma, in, cin, W, H, n, kCM))
    return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(k_conv_igemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
  if (e != cudaSuccess) return e;
  dim3 grid = a.flat ? dim3((unsigned)((n_pos + kCM - 1) / kCM), 1, 1)
                     : dim3((unsigned)((W + kCM - 1) / kCM), (unsigned)H, (unsigned)n);
  k_conv_igemm<<<grid, kConvThreads, kConvSmem, s>>>(ma, mb, a, err);
  return cudaGetLastError();
}

size_t conv_wgrad_part_floats(int cin, int taps, int n, int H, int W) {
  const int n_atoms = taps * (cin / 64), m_tiles = (n_atoms + 1) / 2;
  const int kblocks = n * H * ((W + 63) / 64);
  int per = 0;
  const int splits = wgrad_splits(m_tiles, kblocks, &per);
  return (size_t)splits * m_tiles * 128 * 64;
}

cudaError_t launch_conv_wgrad(const void *in, int cin, int taps, const void *dz, int n, int H,
                              int W, int cout, float *part, size_t part_floats, float *grad,
                              int *err, cudaStream_t s) {
  if (cin < 64 || cin % 64 || (taps != 1 && taps != 9) || n < 1 || H < 1 || W < 1 || cout < 1 ||
      cout > 64 || ((uintptr_t)in & 15) || ((uintptr_t)dz & 15) || !part || !grad)
    return cudaErrorInvalidValue;
  WgradArgs w{};
  w.H = H;
  w.cin_blocks = cin / 64;
  w.taps = taps;
  w.n_atoms = taps * w.cin_blocks;
  w.m_tiles = (w.n_atoms + 1) / 2;
  w.xb = (W + 63) / 64;
  w.kblocks = n * H * w.xb;
  const int splits = wgrad_splits(w.m_tiles, w.kblocks, &w.kb_per_split);
  if ((size_t)splits * w.m_tiles * 128 * 64 > part_floats || w.m_tiles > 65535 || splits > 65535)
    return cudaErrorInvalidValue;
  w.part = part;
  CUtensorMap mx, md;
  if (!tc::make_map_nhwc(&mx, in, cin, W, H, n, 64) || !tc::make_map_nhwc(&md, dz, 64, W, H, n, 64))
    return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kWSmem);
  if (e != cudaSuccess) return e;
  k_conv_wgrad<<<dim3((unsigned)w.m_tiles, (unsigned)splits), kConvThreads, kWSmem, s>>>(mx, md, w,
                                                                                      err);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const int64_t total = (int64_t)cout * taps * cin;
  k_wgrad_reduce<<<grid_for(total, 256), 256, 0, s>>>(part, splits, w.m_tiles, w.cin_blocks, taps,
                                                      cout, grad);
  return cudaGetLastError();
}

cudaError_t launch_bias_grad(const void *dz, int64_t n_pos, int cout, float *part, int part_blocks,
                             float *grad, cudaStream_t s) {
  if (n_pos < 1 || cout < 1 || cout > 64 || part_blocks < 1) return cudaErrorInvalidValue;
  const int64_t chunk = (n_pos + part_blocks - 1) / part_blocks;
  const int nb = (int)((n_pos + chunk - 1) / chunk);
  k_bias_partial<<<nb, 256, 0, s>>>(reinterpret_cast<const __nv_bfloat16 *>(dz), n_pos, chunk, part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_bias_final<<<1, 64, 0, s>>>(part, nb, cout, grad);
  return cudaGetLastError();
}

int loss_blocks(int64_t n_pos) { return (int)((n_pos + 255) / 256); }

cudaError_t launch_loss_grad(const LossArgs &l, void *dz, float *loss_part, double *loss,
                             cudaStream_t s) {
  const int64_t n_pos = (int64_t)l.n * l.H * l.W;
  if (n_pos < 1 || l.P < 1 || l.P > 64) return cudaErrorInvalidValue;
  const int nb = loss_blocks(n_pos);
  k_loss_grad<<<nb, 256, 0, s>>>(l, reinterpret_cast<__nv_bfloat16 *>(dz), loss_part);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_sum_final<<<1, 32, 0, s>>>(loss_part, nb, loss);
  return cudaGetLastError();
}

cudaError_t launch_adam(float *p, const float *g, float *m, float *v, int64_t n, const AdamArgs &a,
                        cudaStream_t s) {
  k_adam<<<grid_for(n, 256), 256, 0, s>>>(p, g, m, v, n, a);
  return cudaGetLastError();
}

cudaError_t launch_pack_weights(const float *params, const PackArgs &a, cudaStream_t s) {
  const int64_t total = (int64_t)64 * a.dim + 8 * (int64_t)64 * 576;
  k_pack_weights<<<grid_for(total, 256), 256, 0, s>>>(params, a);
  return cudaGetLastError();
}

cudaError_t launch_cast_bf16(const float *src, void *dst, int64_t n, cudaStream_t s) {
  if (n % 4 || ((uintptr_t)src & 15) || ((uintptr_t)dst & 7)) return cudaErrorInvalidValue;
  k_cast_bf16<<<grid_for(n / 4, 256), 256, 0, s>>>(reinterpret_cast<const float4 *>(src),
                                                   reinterpret_cast<uint2 *>(dst), n / 4);
  return cudaGetLastError();
}

}  // namespace pa
