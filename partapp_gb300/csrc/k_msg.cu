// k_msg.cu -- pictorial-structures messages on GB300.
//
// One message is computeRotJointMarginal (libPictStruct/
// objectdetect_findrot.cpp:292-456):
//   M    = max(child)                                   (getMinMax, :301-302)
//   J10  = per-rotation nearest shift of child by R(a_r) s offset_c into
//          rotation r + rot_mean_idx, LOG_ZERO outside        (:342-359)
//   E    = exp(J10 - M)                                     (:362-365)
//   E'   = circular rotation filter, clipped taps           (:373-420)
//   J01  = separable truncated Gaussian (x pass, y pass)    (:423-429)
//   out  = nearest shift of log(J01) + M by -R(a_r) s offset_p (:432-448)
// followed by what the caller does with `out` (addGrid2 into the parent
// belief, :637-654; computePartMarginals, :163-236).
//
// Two kernels per batch of independent messages:
//   k_msg_rows  one CTA per (image row y, message): stages all R rotations of
//               the row as exp(J10 - M) in shared memory, applies the rotation
//               filter per column in registers and the x pass along the row,
//               and writes the exp-domain intermediate E2.
//   k_msg_cols_tma  one CTA per (32-column strip, 176-row band, rotation,
//               message): TMA stages the E2 strip with its y halo and the
//               epilogue's inputs, then the y pass (packed FMAs), log, + M,
//               the shift back into the parent frame and the epilogue
//               (store / add / marginal).  k_msg_cols is the same pass with
//               gathered rows, for messages without TMA maps (shift tables
//               that are not plain shifts, widths not a multiple of 4).
// The nearest-shift source indices come from per-message tables computed
// with the reference's double-precision rounding (k_shift_tables).
#include <cuda_bf16.h>

#include "pa_internal.cuh"
#include "tc_common.cuh"

namespace pa {
namespace {

constexpr int kThreadsRows = 384;
constexpr int kThreadsCols = 256;
constexpr int kNO = 11;   // outputs per lane in the row/column passes (odd: conflict-free)
constexpr int kU = 8;     // taps per unrolled block
constexpr int kTX = 32;   // parent columns per k_msg_cols CTA
constexpr int kCW = 33;   // staged source columns (one spare for rounding glitches)
constexpr int kMaxFullTaps = 2048;  // spatial taps of a full-covariance message (sigma <= 341 px)

__device__ __forceinline__ int wrap(int r, int R) { return r < 0 ? r + R : (r >= R ? r - R : r); }

// Packed FP32 FMA (two IEEE fmaf in one instruction, round to nearest, no
// flush to zero): d = a * b + c lane-wise.  The spatial passes accumulate two
// independent output streams per thread with it, so each stream keeps the
// tap order and rounding of a scalar fmaf chain.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

// Asynchronous 4-byte global -> shared copy; `valid` false writes a zero
// and reads nothing (cp.async zero-fill).  All copies of a thread are in
// flight until cp_async_wait_all.
__device__ __forceinline__ void cp_async4(float *smem, const float *gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem),
               "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Source index of a nearest-neighbour shift: a row of the exact table,
// summarised by {c, lo, hi, uniform} when it is the plain shift
// pos -> pos + c on [lo, hi) and -1 elsewhere (always, unless x + t lands
// within an ulp of a half-integer).
__device__ __forceinline__ int shift_src(int4 d, const int16_t *tab, int pos) {
  if (d.w) return (pos >= d.y && pos < d.z) ? pos + d.x : -1;
  return tab[pos];
}

// log of a filtered value: LOG_ZERO for 0 (computeLogGrid).  The accurate
// logf/expf are kept: the approximate intrinsics move near-tied maxima of
// the marginals enough to change the argmax.
__device__ __forceinline__ float log_or_zero(float f) { return f == 0.f ? kLogZero : logf(f); }

// ---------------------------------------------------------------------------
// Rotation filter on columns held in registers: out[r] = sum_j t[j] *
// e[(r - NR + j) mod R] (grid_filter_1d_blas_wraparound,
// libMultiArray/multi_array_filter.hpp:116-155).
// E = exp(J10 - M) and the filter for the columns [x0, x1) of the staged
// pairs E (stride WP), a column per thread at a time; the taps (2 NR + 1)
// stay in registers for all of a thread's columns.  Returns whether an exp
// overflowed.
// ---------------------------------------------------------------------------
template <int R, int NR>
__device__ __forceinline__ bool rot_filter_columns(float2 *E, int WP, int x0, int x1,
                                                   float negM, const float *t) {
  static_assert(R % 2 == 0, "rotation pairs");
  float tv[2 * NR + 1];
#pragma unroll
  for (int j = 0; j < 2 * NR + 1; ++j) tv[j] = t[j];
  float emax = 0.f;
  for (int x = x0 + threadIdx.x; x < x1; x += blockDim.x) {
    float e[R];
#pragma unroll
    for (int p = 0; p < R / 2; ++p) {
      const float2 v = E[p * WP + x];
      e[2 * p] = expf(__fadd_rn(v.x, negM));
      e[2 * p + 1] = expf(__fadd_rn(v.y, negM));
      emax = fmaxf(emax, fmaxf(e[2 * p], e[2 * p + 1]));  // fmaxf skips NaN, as == INF does
    }
    float2 *out = E + x;
#pragma unroll
    for (int q = 0; q < R / 2; ++q) {
      float a0 = 0.f, a1 = 0.f;
#pragma unroll
      for (int j = 0; j < 2 * NR + 1; ++j) {
        a0 = fmaf(tv[j], e[((2 * q - NR + j) % R + R) % R], a0);
        a1 = fmaf(tv[j], e[((2 * q + 1 - NR + j) % R + R) % R], a1);
      }
      out[q * WP] = make_float2(a0, a1);
    }
  }
  return emax == INFINITY;
}

// rot_filter_columns for the runtime half-width nr (one dispatch per tile);
// status bit 1: an exp overflowed, bit 2: nr beyond the specialisations.
template <int R, int NR>
__device__ __forceinline__ int rot_filter_dispatch(int nr, float2 *E, int WP, int x0, int x1,
                                                   float negM, const float *t) {
  if constexpr (NR < 0) {
    return 2;
  } else {
    if (nr == NR) return rot_filter_columns<R, NR>(E, WP, x0, x1, negM, t) ? 1 : 0;
    return rot_filter_dispatch<R, NR - 1>(nr, E, WP, x0, x1, negM, t);
  }
}

// Row stride of the staged rows: left pad covers the widest x kernel, the
// right pad also covers the unrolled tail of the x pass (kU + kNO extra
// reads past the last tap), so every read stays inside zero padding.
__host__ __device__ __forceinline__ int rows_stride(int W, int padx) {
  return W + 2 * padx + kU + kNO;
}

// Shared-memory regions start on 16-byte boundaries (float4 tap loads).
__host__ __device__ __forceinline__ int align4(int n) { return (n + 3) & ~3; }

// ---------------------------------------------------------------------------
// k_msg_rows
//
// Shared layout: rotations are staged in pairs, E2v[p][col] = {E[2p][col],
// E[2p+1][col]} (float2), so one 64-bit load feeds both halves of a packed
// FMA in the x pass.  An odd R gets a zero dummy rotation.
// ---------------------------------------------------------------------------
// One tile of the row pass: image row y, column chunk `chunk` of width cw,
// of message *mdp; kThreadsRows threads; sm: dynamic shared memory of
// rows_smem<RT>(R, cw, padx).
template <int RT>
__device__ __forceinline__ void rows_tile(const MsgDesc *__restrict__ mdp, int Rrt, int H, int W,
                                          int padx, int cw, int y, int chunk, int *err, float *sm) {
  const int R = RT > 0 ? RT : Rrt;
  const int RP = (R + 1) / 2;  // rotation pairs
  const MsgDesc md = *mdp;
  // column chunk [xc0, xc0 + ncw) of the outputs; E holds its columns plus a
  // padx halo on each side (local column lx <-> image column xc0 - padx + lx)
  const int xc0 = chunk * cw;
  const int ncw = min(cw, W - xc0);
  const int WP = rows_stride(cw, padx);
  const int gx0 = max(0, xc0 - padx), gx1 = min(W, xc0 + ncw + padx);  // gathered columns
  const int lg0 = gx0 - xc0 + padx, lg1 = gx1 - xc0 + padx;            // their local range
  const int gw = gx1 - gx0;
  float2 *E = reinterpret_cast<float2 *>(sm);  // [RP][WP] rotation pairs
  const int xpmax = ((2 * padx + 1 + kU - 1) / kU) * kU;
  float2 *tx = E + ((RP * WP + 1) & ~1);     // x taps {t, t}, zero-padded, 16B aligned
  // x taps (none for a full-covariance message: its spatial filter runs on
  // the rotated grid, and the phase's padx does not cover its kernel)
  const int xpad = (md.full || md.tc) ? 0 : ((md.xlen + kU - 1) / kU) * kU;
  float *tr = reinterpret_cast<float *>(tx + xpmax);  // rotation taps
  const int tid = threadIdx.x;

  for (int i = tid; i < xpad; i += blockDim.x) {
    const float t = i < md.xlen ? md.xtaps[i] : 0.f;
    tx[i] = make_float2(t, t);
  }
  for (int i = tid; i < md.rlen; i += blockDim.x) tr[i] = md.rtaps[i];

  // (1) stage exp(J10 - M) for all rotations of row y; zero outside the
  // image (the reference's filter truncates at the border).
  const float negM = -fkey_decode(*md.in_max);
  const int HW = H * W;
  const int npad = WP - gw;
  for (int idx = tid; idx < RP * npad; idx += blockDim.x) {
    const int p = idx / npad, k = idx - p * npad;
    E[p * WP + (k < lg0 ? k : lg1 + (k - lg0))] = make_float2(0.f, 0.f);
  }
  int4 *sdesc = reinterpret_cast<int4 *>(tr + kMaxRot + (RT == 0 ? kThreadsRows * R : 0));
  int *rowoff = reinterpret_cast<int *>(sdesc + 2 * R);  // [R] source row of rotation r, or -1
  float *ostage = reinterpret_cast<float *>(rowoff + align4(R));  // [warps][32 * kNO] output rows
  for (int i = tid; i < 2 * R; i += blockDim.x) sdesc[i] = md.sdesc[i];  // in_x[R], in_y[R]
  __syncthreads();
  for (int r = tid; r < R; r += blockDim.x) {
    const int sy = shift_src(sdesc[R + r], md.ty_in + r * H, y);
    rowoff[r] = sy >= 0 ? (r - md.kidx) * HW + sy * W : -1;
  }
  __syncthreads();
  {
    // Raw child values of the shifted rows land in E by asynchronous copies
    // (all of a thread's copies in flight at once).  Cells without a source
    // get LOG_ZERO, the dummy rotation of an odd R gets -inf (exp -> 0); the
    // exp is taken when the rotation filter reads the column.  A rotation
    // pair p belongs to wpp warps; lane l stages word h = l & 1 (rotation
    // 2p + h) of the pair-cells l >> 1, + 16, ... of its warp's columns, so
    // a warp writes consecutive words and reads the row's shift once.
    float *Ef = reinterpret_cast<float *>(E);
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int h = lane & 1;
    const int wpp = RP >= nwarps ? 1 : nwarps / RP;  // warps per rotation pair
    const int groups = nwarps / wpp;                 // pairs staged at a time
    const int cstep = 16 * wpp;
    if (warp < groups * wpp) {
      for (int p = warp / wpp; p < RP; p += groups) {
        const int r = 2 * p + h;
        float *dst = Ef + ((size_t)p * WP + lg0) * 2 + h;  // pair-cell c at dst[2 c]
        int c = (warp % wpp) * 16 + (lane >> 1);
        const int ro = r < R ? rowoff[r] : -1;
        if (ro < 0) {
          const float fillv = r >= R ? -INFINITY : kLogZero;
          for (; c < gw; c += cstep) dst[2 * c] = fillv;
          continue;
        }
        const int4 d = sdesc[r];
        const float *src = md.in + (int64_t)ro;
        if (d.w) {  // the plain shift gx -> gx + d.x on [d.y, d.z)
          for (; c < gw; c += cstep) {
            const int gx = gx0 + c;
            if (gx >= d.y && gx < d.z) cp_async4(dst + 2 * c, src + gx + d.x, true);
            else dst[2 * c] = kLogZero;
          }
        } else {
          const int16_t *tab = md.tx_in + r * W;
          for (; c < gw; c += cstep) {
            const int sx = tab[gx0 + c];
            if (sx >= 0) cp_async4(dst + 2 * c, src + sx, true);
            else dst[2 * c] = kLogZero;
          }
        }
      }
    }
    cp_async_wait_all();
  }
  __syncthreads();

  // (2) E = exp(J10 - M), then the rotation filter, column by column, in place.
  // rlen < 0: no rotation filter (rot_sigma == 0); rlen == 0: all-zero filter.
  if (md.rlen <= 0) {
    for (int idx = tid; idx < RP * gw; idx += blockDim.x) {
      const int p = idx / gw, x = lg0 + idx - p * gw;
      const float2 v = E[p * WP + x];
      const float2 ev = make_float2(expf(__fadd_rn(v.x, negM)), expf(__fadd_rn(v.y, negM)));
      if (ev.x == INFINITY || ev.y == INFINITY) atomicOr(err, 1);
      E[p * WP + x] = md.rlen == 0 ? make_float2(0.f, 0.f) : ev;
    }
  }
  if (md.rlen > 0) {
    const int nr = (md.rlen - 1) / 2;
    if constexpr (RT > 0) {
      const int bits = rot_filter_dispatch<RT, (RT - 1) / 2>(nr, E, WP, lg0, lg1, negM, tr);
      if (bits) atomicOr(err, bits);
    } else {
      float *col = tr + kMaxRot;  // [blockDim.x][R] scratch
      float *Ef = reinterpret_cast<float *>(E);
      for (int x = lg0 + tid; x < lg1; x += blockDim.x) {
        float *c = col + tid * R;
        for (int r = 0; r < R; ++r) {
          c[r] = expf(__fadd_rn(Ef[((r >> 1) * WP + x) * 2 + (r & 1)], negM));
          if (c[r] == INFINITY) atomicOr(err, 1);
        }
        for (int r = 0; r < R; ++r) {
          float acc = 0.f;
          for (int j = 0; j < md.rlen; ++j) acc = fmaf(tr[j], c[wrap(r - nr + j, R)], acc);
          Ef[((r >> 1) * WP + x) * 2 + (r & 1)] = acc;
        }
      }
    }
  }
  __syncthreads();

  if (md.tc) {
    // tensor-core spatial filter: the rotation-filtered exp map goes out as
    // bf16 rows of the GEMM operand eb [R*H][wp]
    const float *Ef = reinterpret_cast<const float *>(E);
    __nv_bfloat16 *eb = reinterpret_cast<__nv_bfloat16 *>(md.eb);
    for (int idx = tid; idx < R * ncw; idx += blockDim.x) {
      const int r = idx / ncw, j = idx - r * ncw;
      eb[((int64_t)r * H + y) * md.wp + xc0 + j] =
          __float2bfloat16_rn(Ef[((r >> 1) * WP + padx + j) * 2 + (r & 1)]);
    }
    return;
  }
  if (md.full) {
    // full covariance: the rotation-filtered exp map of the chunk goes out
    // as is; the spatial filter runs on the rotated grid (k_full_*)
    const float *Ef = reinterpret_cast<const float *>(E);
    for (int idx = tid; idx < R * ncw; idx += blockDim.x) {
      const int r = idx / ncw, j = idx - r * ncw;
      md.e2[(int64_t)r * HW + (int64_t)y * W + xc0 + j] = Ef[((r >> 1) * WP + padx + j) * 2 + (r & 1)];
    }
    return;
  }

  // (3) x pass over the chunk's outputs: a task is (rotation pair, strip of
  // 32 * kNO columns); lane l owns outputs [l*kNO, l*kNO + kNO) of the strip
  // for both rotations.  The results go through a per-warp shared row so that
  // each store instruction writes 32 consecutive floats.
  const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int kx = (md.xlen - 1) / 2;
  float *e2 = md.e2;
  float *ws = ostage + warp * (32 * kNO);
  const int nstrips = (ncw + 32 * kNO - 1) / (32 * kNO);
  for (int task = warp; task < RP * nstrips; task += nwarps) {
    const int p = task / nstrips;
    const int xs = (task - p * nstrips) * 32 * kNO;  // chunk-relative
    const int x0 = xs + lane * kNO;
    float2 acc[kNO];
#pragma unroll
    for (int i = 0; i < kNO; ++i) acc[i] = make_float2(0.f, 0.f);
    if (x0 < ncw) {
      const float2 *row = E + p * WP + padx - kx + x0;
      for (int kb = 0; kb < xpad; kb += kU) {
        float2 v[kNO + kU - 1];
#pragma unroll
        for (int i = 0; i < kNO + kU - 1; ++i) v[i] = row[kb + i];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const float2 t = tx[kb + u];
#pragma unroll
          for (int i = 0; i < kNO; ++i) acc[i] = ffma2(t, v[i + u], acc[i]);
        }
      }
    }
    const int nx = min(32 * kNO, ncw - xs);
    float *o = e2 + (int64_t)(2 * p) * HW + (int64_t)y * W + xc0 + xs;
    // the staged row goes out in 16-byte words when W is a multiple of 4
    // (then o, HW and nx are too: the chunk and strip starts are multiples of 4)
    auto copy_out = [&](float *dst) {
      if ((W & 3) == 0) {
        const float4 *src4 = reinterpret_cast<const float4 *>(ws);
        float4 *dst4 = reinterpret_cast<float4 *>(dst);
        for (int j = lane; j < (nx >> 2); j += 32) dst4[j] = src4[j];
      } else {
        for (int j = lane; j < nx; j += 32) dst[j] = ws[j];
      }
    };
#pragma unroll
    for (int i = 0; i < kNO; ++i) ws[lane * kNO + i] = acc[i].x;  // odd kNO: conflict-free
    __syncwarp();
    copy_out(o);
    __syncwarp();
    if (2 * p + 1 < R) {
#pragma unroll
      for (int i = 0; i < kNO; ++i) ws[lane * kNO + i] = acc[i].y;
      __syncwarp();
      copy_out(o + HW);
      __syncwarp();
    }
  }
}

// The dynamic shared memory from its first 128-byte boundary (TMA
// destinations start on one); launchers add kSmemAlign bytes.
constexpr int kSmemAlign = 128;
__device__ __forceinline__ float *smem_align128(float *p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  return p + (((kSmemAlign - (a & (kSmemAlign - 1))) & (kSmemAlign - 1)) >> 2);
}

template <int RT>
__global__ void __launch_bounds__(kThreadsRows, RT == 48 ? 1 : 2) k_msg_rows(const MsgDesc *__restrict__ msgs,
                                                           int Rrt, int H, int W, int padx,
                                                           int cw, int *err) {
  extern __shared__ __align__(16) float sm[];
  rows_tile<RT>(msgs + blockIdx.y, Rrt, H, W, padx, cw, (int)blockIdx.x, (int)blockIdx.z, err, sm);
}

// ---------------------------------------------------------------------------
// k_msg_cols
// ---------------------------------------------------------------------------
__device__ __forceinline__ void block_reduce_commit(int key, int *slot, int *sbuf) {
  key = __reduce_max_sync(0xFFFFFFFFu, key);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sbuf[warp] = key;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = sbuf[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = max(m, sbuf[w]);
    atomicMax(slot, m);
  }
  __syncthreads();
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// ---------------------------------------------------------------------------
// Epilogue of a message over the parent cells [y0, y1) x [x0, x1) of
// rotation r: m = log(J01 at the shift-back source) + M, then the caller's
// accumulation (store / add into the parent belief with its max / marginal
// formation with the first-maximum argmax).  getf(sy, sx) returns the
// exp-domain J01 value at source cell (sy, sx).  All threads of the CTA call
// it (block reductions).
// ---------------------------------------------------------------------------
template <class GetF>
__device__ __forceinline__ void msg_epilogue(const MsgDesc &md, int r, int H, int W, int x0,
                                             int x1, int y0, int y1, int4 dxo, int4 dyo,
                                             const int16_t *txo, const int16_t *tyo,
                                             bool first_block, GetF getf, int *red,
                                             unsigned long long *redu) {
  const int tid = threadIdx.x;
  const int64_t HW = (int64_t)H * W;
  const float M = fkey_decode(*md.in_max);
  if (md.in_max_f64 && first_block && tid == 0) *md.in_max_f64 = (double)M;
  const int tw = x1 - x0;
  int k0 = kFkeyNegInf, k1 = kFkeyNegInf;
  unsigned long long am = 0ull;
  const int mode = md.mode;
  const float *src0 = md.src0, *src1 = md.src1;
  float *dst0 = md.dst0, *dst1 = md.dst1;
  // lane = parent column (coalesced row segments), warps step over rows
  const int lx = tid & 31, wy = tid >> 5, nwy = blockDim.x >> 5;
  const int xx = x0 + lx;
  const int sx = lx < tw ? shift_src(dxo, txo, xx) : -1;
  constexpr int U = 4;
  for (int yb = y0 + wy; yb < y1; yb += U * nwy) {
    float m[U], a0[U], a1[U];
    int64_t idx[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int yy = yb + u * nwy;
      idx[u] = -1;
      m[u] = kLogZero;
      a0[u] = 0.f;
      a1[u] = 0.f;
      if (lx < tw && yy < y1) {
        const int sy = shift_src(dyo, tyo, yy);
        if (sy >= 0 && sx >= 0) m[u] = __fadd_rn(log_or_zero(getf(sy, sx)), M);
        idx[u] = (int64_t)r * HW + (int64_t)yy * W + xx;
        if (mode != EPI_STORE) a0[u] = __ldg(src0 + idx[u]);
        if (mode == EPI_DOWN && dst1) a1[u] = __ldg(src1 + idx[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (idx[u] < 0) continue;
      if (mode == EPI_STORE) {
        dst0[idx[u]] = m[u];
      } else if (mode == EPI_ADD) {
        const float o = __fadd_rn(m[u], a0[u]);
        dst0[idx[u]] = o;
        k0 = max(k0, (o == o) ? fkey(o) : kFkeyNegInf);
      } else {
        const float o = __fadd_rn(a0[u], m[u]);
        dst0[idx[u]] = o;
        const unsigned long long k = akey(o, (uint32_t)idx[u]);
        am = k > am ? k : am;
        if (dst1) {
          const float o1 = __fadd_rn(a1[u], m[u]);
          dst1[idx[u]] = o1;
          k1 = max(k1, (o1 == o1) ? fkey(o1) : kFkeyNegInf);
        }
      }
    }
  }
  if (md.mode == EPI_ADD && md.max0) block_reduce_commit(k0, md.max0, red);
  if (md.mode == EPI_DOWN) {
    if (md.max1) block_reduce_commit(k1, md.max1, red);
    if (md.amax0) {
      am = warp_max_u64(am);
      const int lane = tid & 31, warp = tid >> 5;
      if (lane == 0) redu[warp] = am;
      __syncthreads();
      if (tid == 0) {
        unsigned long long bm = redu[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) bm = redu[w] > bm ? redu[w] : bm;
        atomicMax(md.amax0, bm);
      }
    }
  }
}

// The column pass of one (strip, band, rotation) tile of message md with
// the E2 rows gathered by 4-byte asynchronous copies (any shift table).
// sm: the dynamic shared memory of cols_gather_smem(band, pady); red, redu:
// one slot per warp.
__device__ __forceinline__ void cols_gather_tile(const MsgDesc &md, int R, int H, int W, int r,
                                                 int y0, int y1, int x0, int x1, int band,
                                                 int pady, bool first_block, int *err, float *sm,
                                                 int *lim, int *red, unsigned long long *redu) {
  const int tid = threadIdx.x;

  const int16_t *txo = md.tx_out + r * W;
  const int16_t *tyo = md.ty_out + r * H;
  const int4 dxo = md.sdesc[2 * R + r], dyo = md.sdesc[3 * R + r];
  if (tid == 0) {
    lim[0] = 1 << 30; lim[1] = -1; lim[2] = 1 << 30; lim[3] = -1;
    if (dxo.w) {
      const int a = max(x0, dxo.y), b = min(x1, dxo.z);
      if (a < b) { lim[0] = a + dxo.x; lim[1] = b - 1 + dxo.x; }
    }
    if (dyo.w) {
      const int a = max(y0, dyo.y), b = min(y1, dyo.z);
      if (a < b) { lim[2] = a + dyo.x; lim[3] = b - 1 + dyo.x; }
    }
  }
  __syncthreads();
  if (!dxo.w || !dyo.w) {
    int cmn = 1 << 30, cmx = -1, rmn = 1 << 30, rmx = -1;
    for (int i = tid; i < (x1 - x0) + (y1 - y0); i += blockDim.x) {
      if (i < x1 - x0) {
        const int c = dxo.w ? -1 : txo[x0 + i];
        if (c >= 0) { cmn = min(cmn, c); cmx = max(cmx, c); }
      } else {
        const int rr = dyo.w ? -1 : tyo[y0 + i - (x1 - x0)];
        if (rr >= 0) { rmn = min(rmn, rr); rmx = max(rmx, rr); }
      }
    }
    cmn = __reduce_min_sync(0xFFFFFFFFu, cmn);
    cmx = __reduce_max_sync(0xFFFFFFFFu, cmx);
    rmn = __reduce_min_sync(0xFFFFFFFFu, rmn);
    rmx = __reduce_max_sync(0xFFFFFFFFu, rmx);
    if ((tid & 31) == 0) {
      if (!dxo.w) { atomicMin(&lim[0], cmn); atomicMax(&lim[1], cmx); }
      if (!dyo.w) { atomicMin(&lim[2], rmn); atomicMax(&lim[3], rmx); }
    }
  }
  __syncthreads();
  const int cmin = lim[0], cmax = lim[1], rmin = lim[2], rmax = lim[3];
  const bool any = (cmax >= 0 && rmax >= 0);
  const int ky = (md.ylen - 1) / 2;
  const int nrows = any ? rmax - rmin + 1 : 0;      // F rows
  const int srows = nrows + 2 * ky;                  // staged rows
  if (any && (cmax - cmin + 1 > kCW || nrows > band + 2)) {
    if (tid == 0) atomicOr(err, 4);
    return;
  }
  float *S = sm;                                          // [srows + kNO + kU][kCW]
  float *F = S + align4((band + 2 + 2 * pady + kNO + kU) * kCW);  // [nrows][kCW]
  float *ty = F + align4((band + 2) * kCW);               // y taps padded, 16B aligned
  const int ypad = ((md.ylen + kU - 1) / kU) * kU;
  for (int i = tid; i < ypad; i += blockDim.x) ty[i] = i < md.ylen ? md.ytaps[i] : 0.f;

  const int64_t HW = (int64_t)H * W;
  const float *e2 = md.e2 + (int64_t)r * HW;
  if (any) {
    // stage E2 rows [rmin - ky, rmax + ky] x columns [cmin, cmin + kCW), zero
    // outside, by asynchronous copies (all in flight at once); kNO + kU zero
    // rows follow, so the y pass reads its unrolled tail without bounds tests
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    for (int sr = warp; sr < srows + kNO + kU; sr += nwarps) {
      const int yy = rmin - ky + sr;
      const bool rowok = sr < srows && yy >= 0 && yy < H;
      const float *g = e2 + (int64_t)(rowok ? yy : 0) * W + cmin;
      for (int c = lane; c < kCW; c += 32) {
        const bool ok = rowok && cmin + c < W && cmin + c <= cmax;
        cp_async4(S + sr * kCW + c, ok ? g + c : e2, ok);
      }
    }
    cp_async_wait_all();
  }
  __syncthreads();
  if (any) {
    // y pass: lane = column, kNO consecutive rows per lane-task; the row
    // chunks of the 32 strip columns are spread over all warps, the spare
    // column (a strip that needs 33 source columns) gets a second round.
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int ncol = cmax - cmin + 1;
    const int nchunks = (nrows + kNO - 1) / kNO;
    const int ntask = ncol > 32 ? 2 * nchunks : nchunks;
    for (int task = warp; task < ntask; task += nwarps) {
      const int rr0 = (task < nchunks ? task : task - nchunks) * kNO;
      const int c = lane + (task < nchunks ? 0 : 32);
      if (c < ncol) {
        float acc[kNO];
#pragma unroll
        for (int i = 0; i < kNO; ++i) acc[i] = 0.f;
        const float *col = S + c;
        for (int kb = 0; kb < ypad; kb += kU) {
          float v[kNO + kU - 1];
#pragma unroll
          for (int i = 0; i < kNO + kU - 1; ++i) v[i] = col[(rr0 + kb + i) * kCW];
          const float4 ta = *reinterpret_cast<const float4 *>(ty + kb);
          const float4 tb = *reinterpret_cast<const float4 *>(ty + kb + 4);
          const float t[kU] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w};
#pragma unroll
          for (int u = 0; u < kU; ++u)
#pragma unroll
            for (int i = 0; i < kNO; ++i) acc[i] = fmaf(t[u], v[i + u], acc[i]);
        }
#pragma unroll
        for (int i = 0; i < kNO; ++i)
          if (rr0 + i < nrows) F[(rr0 + i) * kCW + c] = acc[i];
      }
    }
  }
  __syncthreads();

  // epilogue: log, + M, shift back, combine with the caller's accumulation.
  msg_epilogue(md, r, H, W, x0, x1, y0, y1, dxo, dyo, txo, tyo, first_block,
               [&](int sy, int sx) { return F[(sy - rmin) * kCW + (sx - cmin)]; }, red, redu);
}

__host__ __device__ __forceinline__ size_t cols_gather_smem(int band, int pady) {
  return ((size_t)align4((band + 2 + 2 * pady + kNO + kU) * kCW) + (size_t)align4((band + 2) * kCW) +
          ((2 * pady + 1 + kU - 1) / kU) * kU) * sizeof(float);
}

__global__ void __launch_bounds__(kThreadsCols) k_msg_cols(const MsgDesc *__restrict__ msgs,
                                                           int R, int H, int W, int band,
                                                           int pady, int *err) {
  const MsgDesc md = msgs[blockIdx.z];
  if (md.full || md.tc) return;  // k_full_* / the tensor-core path (uniform for the CTA)
  const int r = blockIdx.y % R;
  const int yb = blockIdx.y / R;
  const int y0 = yb * band, y1 = min(H, y0 + band);
  const int x0 = blockIdx.x * kTX, x1 = min(W, x0 + kTX);
  extern __shared__ __align__(16) float sm[];
  __shared__ int lim[4];
  __shared__ int red[kThreadsCols / 32];
  __shared__ unsigned long long redu[kThreadsCols / 32];
  cols_gather_tile(md, R, H, W, r, y0, y1, x0, x1, band, pady, blockIdx.x == 0 && blockIdx.y == 0,
                   err, sm, lim, red, redu);
}

// ---------------------------------------------------------------------------
// k_msg_cols_tma: the column pass with the E2 strip staged by TMA.
//
// CTA = 32 parent columns x kCBand rows x one rotation, eight warps.  When
// both shift-back tables of the rotation are plain shifts (the usual case)
// the strip needs source columns [cmin, cmin + 32) and source rows
// [rmin - ky, rmin + nrows + ky) of E2 rotation r: boxes of kCWT x kCBoxRows
// of a 3-D tensor map {W, H, R} at x = floor4(cmin) (16-byte boundary; the
// strip is read from staged column o = cmin mod 4), so rows past the image
// border arrive as zeros -- the reference's truncated filter.  The y pass
// gives each lane one column and two blocks of kNO rows (Dh apart), summed
// with packed FMAs in tap order.  The epilogue takes log, adds M, shifts
// back and combines with the caller's accumulation as msg_epilogue does,
// with 32-bit cell indices.  Other tables take cols_gather_tile.
// ---------------------------------------------------------------------------
constexpr int kColWarps = 8;
constexpr int kColThreads = 32 * kColWarps;
constexpr int kCBand = 2 * kColWarps * kNO;  // 176 rows: one task of 2 x kNO rows per warp
static_assert(kCBand == kColBandRows, "column band of the host's tile count");
constexpr int kCWT = 36;                     // staged columns: 32 + the 16-byte slack
constexpr int kCBoxRows = 64;                // TMA box height
constexpr int kFP = 33;                      // pitch of the filtered tile F

__host__ __device__ __forceinline__ int cols_tma_boxes(int pady) {
  return (kCBand + 2 * pady + kU + kCBoxRows - 1) / kCBoxRows;
}
// offset (floats) of the epilogue input tiles src0 / src1 [kCBand][kTX]
// each, 128-byte aligned after the E2 tile, F and the y taps
__host__ __device__ __forceinline__ size_t cols_src_off(int pady) {
  const size_t o = (size_t)cols_tma_boxes(pady) * kCBoxRows * kCWT + (size_t)kCBand * kFP +
                   ((2 * pady + 1 + kU - 1) / kU) * kU;
  return (o + 31) / 32 * 32;
}
__host__ __device__ __forceinline__ size_t cols_tma_smem(int pady) {
  const size_t tile = cols_src_off(pady) + (size_t)2 * kCBand * kTX;
  const size_t g = cols_gather_smem(kCBand, pady) / sizeof(float);
  return (tile > g ? tile : g) * sizeof(float) + kSmemAlign;
}

// One tile of the column pass: strip bx, (band, rotation) index by of
// message *mdp (kTX columns x kCBand rows x one rotation); any multiple of
// 32 threads up to 1024; sm: 128-byte aligned shared memory of
// cols_tma_smem(pady) (less the alignment slack).  The barriers are
// invalidated at the end, so that a persistent CTA can run tile after tile.
__device__ __forceinline__ void cols_tile_tma(const MsgDesc *__restrict__ mdp, int R, int H, int W,
                                              int pady, int bx, int by, int *err, float *sm) {
  const MsgDesc md = *mdp;
  if (md.full || md.tc) return;
  const int r = by % R;
  const int y0 = (by / R) * kCBand, y1 = min(H, y0 + kCBand);
  const int x0 = bx * kTX, x1 = min(W, x0 + kTX);
  const bool first_block = bx == 0 && by == 0;
  const int nw = blockDim.x >> 5;
  __shared__ int lim[4];
  __shared__ int red[32];
  __shared__ unsigned long long redu[32];
  __shared__ __align__(8) uint64_t bar, bar_src;
  const int4 dxo = md.sdesc[2 * R + r], dyo = md.sdesc[3 * R + r];
  if (!dxo.w || !dyo.w) {  // uniform for the CTA
    cols_gather_tile(md, R, H, W, r, y0, y1, x0, x1, kCBand, pady, first_block, err, sm, lim, red,
                     redu);
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // parent cells with a source: columns [xa, xb), rows [ya, yb)
  const int xa = max(x0, dxo.y), xb = min(x1, dxo.z);
  const int ya = max(y0, dyo.y), yb = min(y1, dyo.z);
  const bool any = xa < xb && ya < yb;
  const int cmin = xa + dxo.x, rmin = ya + dyo.x, nrows = any ? yb - ya : 0;
  const int ky = (md.ylen - 1) / 2;
  const int Dh = ((nrows + 1) / 2 + kNO - 1) / kNO * kNO;  // second row block's offset
  const int nb = (2 * Dh + 2 * ky + kU + kCBoxRows - 1) / kCBoxRows;
  float *S = sm;                                               // [nb * kCBoxRows][kCWT]
  float *F = S + (size_t)cols_tma_boxes(pady) * kCBoxRows * kCWT;  // [kCBand][kFP]
  float *ty = F + kCBand * kFP;
  float *S0 = sm + cols_src_off(pady), *S1 = S0 + kCBand * kTX;  // [kCBand][kTX] each
  const int ypad = ((md.ylen + kU - 1) / kU) * kU;
  const int nsrc = md.mode == EPI_STORE ? 0 : (md.mode == EPI_DOWN && md.dst1 ? 2 : 1);
  for (int i = tid; i < ypad; i += blockDim.x) ty[i] = i < md.ylen ? md.ytaps[i] : 0.f;
  const int xs0 = cmin & ~3, o = cmin - xs0;
  // TMA wants 128-byte aligned destinations and a 64-byte aligned map: a
  // violation is reported (error bit 16) and the tile is not staged
  const bool tma_ok = (tc::smem_u32(S) & 127u) == 0 && (tc::smem_u32(S0) & 127u) == 0 &&
                      ((uintptr_t)md.tm_e2 & 63u) == 0 && ((uintptr_t)md.tm_src0 & 63u) == 0 &&
                      ((uintptr_t)md.tm_src1 & 63u) == 0 && (nsrc < 1 || md.tm_src0) &&
                      (nsrc < 2 || md.tm_src1);
  if (!tma_ok && tid == 0) atomicOr(err, 16);
  if (tma_ok && tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_init(&bar_src, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (any) {
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(md.tm_e2) : "memory");
      tc::mbar_arrive_expect_tx(&bar, (uint32_t)(nb * kCBoxRows * kCWT * 4));
      for (int b = 0; b < nb; ++b)
        tc::tma_load_3d(S + (size_t)b * kCBoxRows * kCWT, md.tm_e2, xs0, rmin - ky + b * kCBoxRows,
                        r, &bar);
    }
    // the epilogue's inputs arrive while the y pass runs
    tc::mbar_arrive_expect_tx(&bar_src, (uint32_t)(nsrc * kCBand * kTX * 4));
    for (int k = 0; k < nsrc; ++k) {
      const CUtensorMap *m = k ? md.tm_src1 : md.tm_src0;
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
      tc::tma_load_3d(k ? S1 : S0, m, x0, y0, r, &bar_src);
    }
  }
  // thread 0 watches the copies (bounded); the barrier then hands the tile
  // to the CTA, and a run-out wait sends the whole CTA home (error bit set)
  __shared__ int s_ok;
  if (tid == 0) {
    s_ok = !tma_ok ? 0 : any ? (int)tc::mbar_wait_try(&bar, 0, err) : 1;
    if (!s_ok && tma_ok) {  // once more for the copies in flight
      tc::mbar_wait_try(&bar, 0, err);
      tc::mbar_wait_try(&bar_src, 0, err);
    }
  }
  __syncthreads();
  if (!s_ok) {
    if (tid == 0 && tma_ok) {
      tc::mbar_inval(&bar);
      tc::mbar_inval(&bar_src);
    }
    return;
  }
  // y pass: warp w, lane c -> column c, rows [w*kNO, w*kNO + kNO) and the
  // same rows + Dh
  const int ncol = xb - xa;
  for (int t = warp; t * kNO < Dh; t += nw) {
    const int q0 = t * kNO;
    float2 acc[kNO];
#pragma unroll
    for (int i = 0; i < kNO; ++i) acc[i] = make_float2(0.f, 0.f);
    const float *col = S + o + lane;
    for (int kb = 0; kb < ypad; kb += kU) {
      float2 v[kNO + kU - 1];
#pragma unroll
      for (int i = 0; i < kNO + kU - 1; ++i)
        v[i] = make_float2(col[(q0 + kb + i) * kCWT], col[(q0 + Dh + kb + i) * kCWT]);
      const float4 ta = *reinterpret_cast<const float4 *>(ty + kb);
      const float4 tb = *reinterpret_cast<const float4 *>(ty + kb + 4);
      const float tt[kU] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w};
#pragma unroll
      for (int u = 0; u < kU; ++u)
#pragma unroll
        for (int i = 0; i < kNO; ++i) acc[i] = ffma2(make_float2(tt[u], tt[u]), v[i + u], acc[i]);
    }
    if (lane < ncol) {
#pragma unroll
      for (int i = 0; i < kNO; ++i) {
        if (q0 + i < nrows) F[(q0 + i) * kFP + lane] = acc[i].x;
        if (q0 + Dh + i < nrows) F[(q0 + Dh + i) * kFP + lane] = acc[i].y;
      }
    }
  }
  // a second word: a slow warp may still be reading s_ok from the first test
  __shared__ int s_src_ok;
  if (tid == 0) {
    s_src_ok = 1;
    if (!tc::mbar_wait_try(&bar_src, 0, err)) {
      tc::mbar_wait_try(&bar_src, 0, err);  // once more for the copies in flight
      s_src_ok = 0;
    }
  }
  __syncthreads();
  if (!s_src_ok) {
    if (tid == 0) {
      tc::mbar_inval(&bar);
      tc::mbar_inval(&bar_src);
    }
    return;
  }

  // epilogue (msg_epilogue's arithmetic for plain shifts), inputs from S0 / S1
  const float M = fkey_decode(*md.in_max);
  if (md.in_max_f64 && first_block && tid == 0) *md.in_max_f64 = (double)M;
  const int HW = H * W;
  const int xx = x0 + lane;
  const bool colin = xx < x1;
  const bool colok = colin && xx >= xa && xx < xb;
  const int fc = xx - xa;  // F column of xx (source column xx + dxo.x - cmin)
  const int mode = md.mode;
  float *dst0 = md.dst0, *dst1 = md.dst1;
  int k0 = kFkeyNegInf, k1 = kFkeyNegInf;
  unsigned long long am = 0ull;
  // One loop per mode (uniform for the CTA).  The running maxima are keyed
  // as before; a cell below the current maximum as a float (never true for
  // NaN) cannot change its key and skips the key arithmetic.
  if (colin) {
    auto mval = [&](int yy) {
      return (colok && yy >= ya && yy < yb) ? __fadd_rn(log_or_zero(F[(yy - ya) * kFP + fc]), M)
                                            : kLogZero;
    };
    const int didx = nw * W, dsi = nw * kTX;
    int idx = r * HW + (y0 + warp) * W + xx, si = warp * kTX + lane;
    if (mode == EPI_STORE) {
#pragma unroll 4
      for (int yy = y0 + warp; yy < y1; yy += nw, idx += didx) dst0[idx] = mval(yy);
    } else if (mode == EPI_ADD) {
      float b0 = -INFINITY;
#pragma unroll 4
      for (int yy = y0 + warp; yy < y1; yy += nw, idx += didx, si += dsi) {
        const float ov = __fadd_rn(mval(yy), S0[si]);
        dst0[idx] = ov;
        if (!(ov < b0)) {
          const int k = (ov == ov) ? fkey(ov) : kFkeyNegInf;
          if (k > k0) k0 = k, b0 = ov;
        }
      }
    } else {
      float ba = -INFINITY, b1 = -INFINITY;
#pragma unroll 4
      for (int yy = y0 + warp; yy < y1; yy += nw, idx += didx, si += dsi) {
        const float m = mval(yy);
        const float ov = __fadd_rn(S0[si], m);
        dst0[idx] = ov;
        if (!(ov < ba)) {
          const unsigned long long k = akey(ov, (uint32_t)idx);
          if (k > am) {
            am = k;
            if (ov == ov) ba = ov;  // a NaN's key is the lowest: it never raises the filter
          }
        }
        if (dst1) {
          const float o1 = __fadd_rn(S1[si], m);
          dst1[idx] = o1;
          if (!(o1 < b1)) {
            const int k = (o1 == o1) ? fkey(o1) : kFkeyNegInf;
            if (k > k1) k1 = k, b1 = o1;
          }
        }
      }
    }
  }
  if (mode == EPI_ADD && md.max0) block_reduce_commit(k0, md.max0, red);
  if (mode == EPI_DOWN) {
    if (md.max1) block_reduce_commit(k1, md.max1, red);
    if (md.amax0) {
      am = warp_max_u64(am);
      if (lane == 0) redu[warp] = am;
      __syncthreads();
      if (tid == 0) {
        unsigned long long bm = redu[0];
        for (int w = 1; w < nw; ++w) bm = redu[w] > bm ? redu[w] : bm;
        atomicMax(md.amax0, bm);
      }
    }
  }
  __syncthreads();  // the reductions' shared words are read before the next tile
  if (tid == 0) {
    tc::mbar_inval(&bar);
    tc::mbar_inval(&bar_src);
  }
}

__global__ void __launch_bounds__(kColThreads, 2) k_msg_cols_tma(const MsgDesc *__restrict__ msgs,
                                                              int R, int H, int W, int pady,
                                                              int *err) {
  extern __shared__ __align__(16) float sm_raw[];
  cols_tile_tma(msgs + blockIdx.z, R, H, W, pady, (int)blockIdx.x, (int)blockIdx.y, err,
                smem_align128(sm_raw));
}

// ---------------------------------------------------------------------------
// Full-covariance messages: gaussFilter2dOffset with a zero offset
// (libMultiArray/multi_array_filter.hpp:335-369) on every rotation of the
// rotation-filtered exp map e2: bilinear rotation into the eigenbasis of C
// (transform_grid_resize), unnormalised truncated Gaussians along the eigen
// axes (gaussFilterDiag2d), bilinear rotation back
// (transform_grid_fixed_size), then the usual log / + M / shift-back
// epilogue.  Coordinates are evaluated in double with the reference's
// rounding, bilinear weights in float (explicit _rn operations: no fused
// multiply-add).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void map_pt(const double *T, int x, int y, double &ox, double &oy) {
  ox = __dadd_rn(__dadd_rn(__dmul_rn(T[0], (double)x), __dmul_rn(T[1], (double)y)), T[2]);
  oy = __dadd_rn(__dadd_rn(__dmul_rn(T[3], (double)x), __dmul_rn(T[4], (double)y)), T[5]);
}

// TM_BILINEAR sample of g [in_h][in_w] (multi_array_transform.hpp:216-236):
// exact-hit shortcut, last row/column and outside left at 0.
__device__ __forceinline__ float bilinear_at(const float *g, int in_h, int in_w, double x1,
                                             double y1) {
  const double fx = floor(x1), fy = floor(y1);
  if (!(fx >= 0.0 && fx < (double)in_w && fy >= 0.0 && fy < (double)in_h)) return 0.f;
  const int ix1 = (int)fx, iy1 = (int)fy;
  const float a = __double2float_rn(__dsub_rn(x1, fx));
  const float b = __double2float_rn(__dsub_rn(y1, fy));
  const float eps10 = 10.0f * 1.1920928955078125e-07f;  // 10 * FLT_EPSILON
  const float *g0 = g + (int64_t)iy1 * in_w + ix1;
  if (a < eps10 && b < eps10) return __ldg(g0);
  if (ix1 >= in_w - 1 || iy1 >= in_h - 1) return 0.f;
  const float *g1 = g0 + in_w;
  const float omb = __fsub_rn(1.0f, b), oma = __fsub_rn(1.0f, a);
  const float t0 = __fmul_rn(__fmul_rn(omb, oma), __ldg(g0));
  const float t1 = __fmul_rn(__fmul_rn(omb, a), __ldg(g0 + 1));
  const float t2 = __fmul_rn(__fmul_rn(b, oma), __ldg(g1));
  const float t3 = __fmul_rn(__fmul_rn(b, a), __ldg(g1 + 1));
  return __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
}

// e2 [R][H][W] -> g0 [R][oh][ow] (bilinear; sparse messages take k_full_d*)
__global__ void __launch_bounds__(256) k_full_fwd(const MsgDesc *__restrict__ msgs, int R, int H,
                                                  int W) {
  const int msg = blockIdx.z / R, r = blockIdx.z - (blockIdx.z / R) * R;
  const MsgDesc *md = msgs + msg;
  if (!md->full || md->sparse) return;
  const int oh = md->oh, ow = md->ow;
  const int x3 = blockIdx.x * 32 + threadIdx.x, y3 = blockIdx.y * 8 + threadIdx.y;
  if (x3 >= ow || y3 >= oh) return;
  double x1, y1;
  map_pt(md->tf, x3, y3, x1, y1);
  md->g0[((int64_t)r * oh + y3) * ow + x3] =
      bilinear_at(md->e2 + (int64_t)r * H * W, H, W, x1, y1);
}

// TM_DIRECT forward rotation (bIsSparse): every e2 cell that is not 0 lands
// on its nearest g0 cell, the last one in the reference's loop order (x
// outer, y inner) winning; cells no input reaches stay 0.  g1 (free until the
// x pass) holds, per g0 cell, 1 + the enumeration index of its winner.
__global__ void __launch_bounds__(256) k_full_dclear(const MsgDesc *__restrict__ msgs, int R) {
  const int msg = blockIdx.z / R, r = blockIdx.z - (blockIdx.z / R) * R;
  const MsgDesc *md = msgs + msg;
  if (!md->full || !md->sparse) return;
  const int x3 = blockIdx.x * 32 + threadIdx.x, y3 = blockIdx.y * 8 + threadIdx.y;
  if (x3 >= md->ow || y3 >= md->oh) return;
  reinterpret_cast<int *>(md->g1)[((int64_t)r * md->oh + y3) * md->ow + x3] = 0;
}

__global__ void __launch_bounds__(256) k_full_dscatter(const MsgDesc *__restrict__ msgs, int R,
                                                       int H, int W) {
  const int msg = blockIdx.z / R, r = blockIdx.z - (blockIdx.z / R) * R;
  const MsgDesc *md = msgs + msg;
  if (!md->full || !md->sparse) return;
  const int x1 = blockIdx.x * 32 + threadIdx.x, y1 = blockIdx.y * 8 + threadIdx.y;
  if (x1 >= W || y1 >= H) return;
  if (md->e2[((int64_t)r * H + y1) * W + x1] == 0.f) return;  // the default is not mapped
  double x3, y3;
  map_pt(md->td, x1, y1, x3, y3);
  const double fx = floor(__dadd_rn(x3, 0.5)), fy = floor(__dadd_rn(y3, 0.5));
  if (!(fx >= 0.0 && fx < (double)md->ow && fy >= 0.0 && fy < (double)md->oh)) return;
  const int e = x1 * H + y1 + 1;  // enumeration order of the reference's loops, 1-based
  atomicMax(reinterpret_cast<int *>(md->g1) + ((int64_t)r * md->oh + (int)fy) * md->ow + (int)fx, e);
}

__global__ void __launch_bounds__(256) k_full_dgather(const MsgDesc *__restrict__ msgs, int R,
                                                      int H, int W) {
  const int msg = blockIdx.z / R, r = blockIdx.z - (blockIdx.z / R) * R;
  const MsgDesc *md = msgs + msg;
  if (!md->full || !md->sparse) return;
  const int x3 = blockIdx.x * 32 + threadIdx.x, y3 = blockIdx.y * 8 + threadIdx.y;
  if (x3 >= md->ow || y3 >= md->oh) return;
  const int64_t o = ((int64_t)r * md->oh + y3) * md->ow + x3;
  const int e = reinterpret_cast<const int *>(md->g1)[o];
  float v = 0.f;
  if (e > 0) {
    const int x1 = (e - 1) / H, y1 = (e - 1) - x1 * H;
    v = md->e2[((int64_t)r * H + y1) * W + x1];
  }
  md->g0[o] = v;
}

// x pass along the rotated rows: g0 -> g1 (truncated at the border)
__global__ void __launch_bounds__(256) k_full_gx(const MsgDesc *__restrict__ msgs, int R) {
  const MsgDesc *md = msgs + blockIdx.z;
  if (!md->full) return;
  const int oh = md->oh, ow = md->ow, r = blockIdx.y, y = blockIdx.x;
  if (y >= oh) return;  // uniform for the CTA
  const int xlen = md->xlen, kx = (xlen - 1) / 2;
  extern __shared__ __align__(16) float sm[];
  float *t = sm;                 // [xlen]
  float *row = sm + align4(xlen);  // [ow + 2 kx], zero outside the grid
  for (int i = threadIdx.x; i < xlen; i += blockDim.x) t[i] = md->xtaps[i];
  const float *src = md->g0 + ((int64_t)r * oh + y) * ow;
  for (int i = threadIdx.x; i < ow + 2 * kx; i += blockDim.x) {
    const int x = i - kx;
    row[i] = (x >= 0 && x < ow) ? __ldg(src + x) : 0.f;
  }
  __syncthreads();
  float *dst = md->g1 + ((int64_t)r * oh + y) * ow;
  for (int x = threadIdx.x; x < ow; x += blockDim.x) {
    float acc = 0.f;
    for (int k = 0; k < xlen; ++k) acc = fmaf(t[k], row[x + k], acc);
    dst[x] = acc;
  }
}

// y pass along the rotated columns: g1 -> g0 (truncated at the border)
constexpr int kFullRows = 32;
__global__ void __launch_bounds__(256) k_full_gy(const MsgDesc *__restrict__ msgs, int R) {
  const int msg = blockIdx.z / R, r = blockIdx.z - (blockIdx.z / R) * R;
  const MsgDesc *md = msgs + msg;
  if (!md->full) return;
  const int oh = md->oh, ow = md->ow;
  const int ylen = md->ylen, ky = (ylen - 1) / 2;
  __shared__ float t[kMaxFullTaps];
  for (int i = threadIdx.y * 32 + threadIdx.x; i < ylen; i += 256) t[i] = md->ytaps[i];
  __syncthreads();
  const int x = blockIdx.x * 32 + threadIdx.x;
  if (x >= ow) return;
  const float *src = md->g1 + (int64_t)r * oh * ow + x;
  float *dst = md->g0 + (int64_t)r * oh * ow + x;
  const int yend = min(oh, (blockIdx.y + 1) * kFullRows);
  for (int y = blockIdx.y * kFullRows + threadIdx.y; y < yend; y += 8) {
    const int k0 = max(0, ky - y), k1 = min(ylen, oh - y + ky);
    float acc = 0.f;
    for (int k = k0; k < k1; ++k) acc = fmaf(t[k], __ldg(src + (int64_t)(y - ky + k) * ow), acc);
    dst[(int64_t)y * ow] = acc;
  }
}

// rotate back (bilinear from g0 at tb * (x, y)), log, + M, shift back, epilogue
constexpr int kFullBand = 64;
__global__ void __launch_bounds__(kThreadsCols) k_full_epi(const MsgDesc *__restrict__ msgs, int R,
                                                          int H, int W) {
  __shared__ int red[kThreadsCols / 32];
  __shared__ unsigned long long redu[kThreadsCols / 32];
  const MsgDesc md = msgs[blockIdx.z];
  if (!md.full) return;
  const int r = blockIdx.y % R, yb = blockIdx.y / R;
  const int y0 = yb * kFullBand, y1 = min(H, y0 + kFullBand);
  const int x0 = blockIdx.x * kTX, x1 = min(W, x0 + kTX);
  const int16_t *txo = md.tx_out + r * W;
  const int16_t *tyo = md.ty_out + r * H;
  const int4 dxo = md.sdesc[2 * R + r], dyo = md.sdesc[3 * R + r];
  const float *g = md.g0 + (int64_t)r * md.oh * md.ow;
  const int oh = md.oh, ow = md.ow;
  msg_epilogue(md, r, H, W, x0, x1, y0, y1, dxo, dyo, txo, tyo, blockIdx.x == 0 && blockIdx.y == 0,
               [&](int sy, int sx) {
                 double px, py;
                 map_pt(md.tb, sx, sy, px, py);
                 return bilinear_at(g, oh, ow, px, py);
               },
               red, redu);
}

// ---------------------------------------------------------------------------
// Tensor-core spatial filter (large grids): the truncated separable Gaussian
// as two banded Toeplitz products on tcgen05 (k_tc_gemm.cu).  T[i][j] =
// t[j - i + k] for |j - i| <= k, 0 elsewhere, in bf16; the reference's
// truncation at the border is the Toeplitz matrix restricted to the grid.
// ---------------------------------------------------------------------------
__global__ void k_tc_toeplitz(const MsgDesc *__restrict__ msgs, int H, int W) {
  const MsgDesc *md = msgs + blockIdx.y;
  if (!md->tc) return;
  const int kx = (md->xlen - 1) / 2, ky = (md->ylen - 1) / 2;
  __nv_bfloat16 *tx = reinterpret_cast<__nv_bfloat16 *>(md->tbx);
  __nv_bfloat16 *ty = reinterpret_cast<__nv_bfloat16 *>(md->tby);
  const int64_t nx = (int64_t)W * md->wp, ny = (int64_t)H * md->hp;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nx + ny;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < nx) {
      const int r = (int)(i / md->wp), c = (int)(i - (int64_t)r * md->wp), d = c - r;
      tx[i] = __float2bfloat16_rn((d >= -kx && d <= kx && c < W) ? md->xtaps[d + kx] : 0.f);
    } else {
      const int64_t k = i - nx;
      const int r = (int)(k / md->hp), c = (int)(k - (int64_t)r * md->hp), d = c - r;
      ty[k] = __float2bfloat16_rn((d >= -ky && d <= ky && c < H) ? md->ytaps[d + ky] : 0.f);
    }
  }
}

__global__ void __launch_bounds__(kThreadsCols) k_tc_epi(const MsgDesc *__restrict__ msgs, int R,
                                                        int H, int W) {
  __shared__ int red[kThreadsCols / 32];
  __shared__ unsigned long long redu[kThreadsCols / 32];
  const MsgDesc md = msgs[blockIdx.z];
  if (!md.tc) return;
  const int r = blockIdx.y % R, yb = blockIdx.y / R;
  const int y0 = yb * kFullBand, y1 = min(H, y0 + kFullBand);
  const int x0 = blockIdx.x * kTX, x1 = min(W, x0 + kTX);
  const int16_t *txo = md.tx_out + r * W;
  const int16_t *tyo = md.ty_out + r * H;
  const int4 dxo = md.sdesc[2 * R + r], dyo = md.sdesc[3 * R + r];
  const float *yv = md.yv + (int64_t)r * H * W;
  msg_epilogue(md, r, H, W, x0, x1, y0, y1, dxo, dyo, txo, tyo, blockIdx.x == 0 && blockIdx.y == 0,
               [&](int sy, int sx) { return __ldg(yv + (int64_t)sy * W + sx); }, red, redu);
}

// ---------------------------------------------------------------------------
// Shift tables: the nearest-neighbour source index of
// transform_grid_fixed_size with a pure translation
// (multi_array_transform.hpp:194-215): floor((x3 + a) + 0.5), -1 outside.
// shifts[msg][4][R] = {a_x_in, a_y_in, a_x_out, a_y_out}; NaN in a_*_in marks
// a log_joint_10 rotation without a source rotation.
// tables[msg] = tx_in[R][W], ty_in[R][H], tx_out[R][W], ty_out[R][H].
// ---------------------------------------------------------------------------
__global__ void k_shift_tables(const double *__restrict__ shifts, int R, int H, int W,
                               int16_t *__restrict__ tables) {
  const int msg = blockIdx.y;
  const double *sh = shifts + (size_t)msg * 4 * R;
  int16_t *tb = tables + (size_t)msg * 2 * R * (W + H);
  const int per = R * (W + H);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * per; i += gridDim.x * blockDim.x) {
    const int side = i / per;  // 0: in, 1: out
    int j = i - side * per;
    int r, pos, n, axis;
    if (j < R * W) {
      r = j / W; pos = j - r * W; n = W; axis = 0;
    } else {
      j -= R * W;
      r = j / H; pos = j - r * H; n = H; axis = 1;
    }
    const double a = sh[(side * 2 + axis) * R + r];
    int16_t v = -1;
    if (a == a) {
      const double p = __dadd_rn(__dadd_rn((double)pos, a), 0.5);
      const double f = floor(p);
      if (f >= 0.0 && f < (double)n) v = (int16_t)f;
    }
    // layout: side 0 -> [tx_in | ty_in], side 1 -> [tx_out | ty_out]
    tb[side * per + (axis == 0 ? r * W + pos : R * W + r * H + pos)] = v;
  }
}

// Summaries {c, lo, hi, uniform} of every table row.  sdesc[msg] =
// [in_x[R] | in_y[R] | out_x[R] | out_y[R]].
__global__ void k_shift_desc(const int16_t *__restrict__ tables, int n_msgs, int R, int H, int W,
                             int4 *__restrict__ sdesc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_msgs * 4 * R) return;
  const int msg = i / (4 * R), k = i - msg * 4 * R;
  const int which = k / R, r = k - which * R;  // 0 in_x, 1 in_y, 2 out_x, 3 out_y
  const int n = (which & 1) ? H : W;
  const int16_t *tb = tables + (size_t)msg * 2 * R * (W + H) + (which >= 2 ? (size_t)R * (W + H) : 0) +
                      ((which & 1) ? (size_t)R * W + (size_t)r * H : (size_t)r * W);
  int lo = -1, hi = -1, c = 0;
  bool uniform = true;
  for (int p = 0; p < n; ++p) {
    const int v = tb[p];
    if (v >= 0) {
      if (lo < 0) { lo = p; c = v - p; }
      else if (hi >= 0 || v != p + c) uniform = false;  // a gap or a different shift
    } else if (lo >= 0 && hi < 0) {
      hi = p;
    }
  }
  if (lo < 0) { lo = 0; hi = 0; }
  else if (hi < 0) hi = n;
  sdesc[i] = make_int4(c, lo, hi, uniform ? 1 : 0);
}

template <int RT>
size_t rows_smem(int R, int cw, int padx) {
  const int WP = rows_stride(cw, padx);
  const int RP = (R + 1) / 2;
  size_t smem = ((size_t)2 * ((RP * WP + 1) & ~1) + 2 * ((2 * padx + 1 + kU - 1) / kU) * kU + kMaxRot) *
                sizeof(float);
  if (RT == 0) smem += (size_t)kThreadsRows * R * sizeof(float);
  smem += (size_t)2 * R * sizeof(int4) + (size_t)align4(R) * sizeof(int) +
          (size_t)(kThreadsRows / 32) * 32 * kNO * sizeof(float);
  return smem;
}

// Column chunk of the row kernel: the whole row when two CTAs fit on an SM
// (one for R = 48), else the widest chunk that does (a multiple of 32 * kNO
// outputs, at least one strip), else the widest that fits at all.
template <int RT>
int rows_chunk(int R, int W, int padx) {
  const size_t target = (RT == 48 ? 227 : 113) * 1024;
  if (rows_smem<RT>(R, W, padx) <= target) return W;
  for (size_t lim : {target, (size_t)227 * 1024}) {
    int best = 0;
    for (int cw = 32 * kNO; cw < W; cw += 32 * kNO)
      if (rows_smem<RT>(R, cw, padx) <= lim) best = cw;
    if (best) return best;
  }
  return 0;
}

template <int RT>
cudaError_t launch_rows_t(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int padx,
                          int *err, cudaStream_t s, int cw_force = 0) {
  const int cw = cw_force > 0 ? cw_force : rows_chunk<RT>(R, W, padx);
  if (cw <= 0 || (int64_t)R * H * W >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  const size_t smem = rows_smem<RT>(R, cw, padx);
  cudaFuncSetAttribute(k_msg_rows<RT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid((unsigned)H, (unsigned)n_msgs, (unsigned)((W + cw - 1) / cw));
  k_msg_rows<RT><<<grid, kThreadsRows, smem, s>>>(msgs, R, H, W, padx, cw, err);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// k_ps_queue: message passing of many images (sizes and rotation counts may
// differ) in one persistent launch.
//
// Every CTA takes the next tile index from a global head (atomicAdd), finds
// its job (binary search over the jobs' first tiles), waits until the jobs
// it depends on are complete, runs the tile, and counts it done.  The host
// orders the jobs so that every dependency points to an earlier job: the
// upward row and column jobs level by level (post-order), the root
// combinations, then the downward ones (pre-order).  A CTA waits only for
// tiles taken before its own, by CTAs that are running and wait only for
// earlier tiles in turn, so the queue cannot deadlock whatever number of
// CTAs is resident.  Waits are bounded in time (globaltimer): on expiry the
// CTA sets status bit 1 and the whole launch stops taking tiles.
//
// Memory order: every thread fences its tile's writes before the barrier
// that precedes the done-count; the waiting thread reads counts with
// acquire semantics and orders them before the TMA loads of the next tile
// (fence.proxy.async), which read the maps other CTAs wrote.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The 48-rotation row tile holds a whole column of 48 values in registers;
// kept out of line, its register spills stay inside its own tiles.
__device__ __noinline__ void rows_tile_48(const MsgDesc *md, int H, int W, int padx, int cw, int y,
                                          int chunk, int *err, float *sm) {
  rows_tile<48>(md, 48, H, W, padx, cw, y, chunk, err, sm);
}
__device__ __noinline__ void rows_tile_any(const MsgDesc *md, int R, int H, int W, int padx,
                                           int cw, int y, int chunk, int *err, float *sm) {
  rows_tile<0>(md, R, H, W, padx, cw, y, chunk, err, sm);
}

__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// One tile t of job j.
__device__ __forceinline__ void ps_queue_tile(const QJob &j, int t, int *err, float *sm) {
  if (j.type == QJOB_ROWS) {
    const int y = t / j.nch, chunk = t - (t / j.nch) * j.nch;
    switch (j.R) {
      case 12: rows_tile<12>(j.md, j.R, j.H, j.W, j.pad, j.cw, y, chunk, err, sm); break;
      case 24: rows_tile<24>(j.md, j.R, j.H, j.W, j.pad, j.cw, y, chunk, err, sm); break;
      case 48: rows_tile_48(j.md, j.H, j.W, j.pad, j.cw, y, chunk, err, sm); break;
      default: rows_tile_any(j.md, j.R, j.H, j.W, j.pad, j.cw, y, chunk, err, sm); break;
    }
  } else if (j.type == QJOB_COLS) {
    cols_tile_tma(j.md, j.R, j.H, j.W, j.pad, t % j.nch, t / j.nch, err, sm);
  } else if (j.type == QJOB_ROOT) {
    const long long c0 = (long long)t * kQRootCells;
    root_combine_cells<kQMaxDeps, 4>(*j.rd, c0, min(j.cells, c0 + kQRootCells), blockDim.x);
  }
}

__global__ void __launch_bounds__(kQThreads, 2)
    k_ps_queue(const QJob *__restrict__ jobs, int n_jobs, long long n_items,
               unsigned long long *head, int *done, int *status, int *err, long long wait_limit_ns,
               unsigned long long *stats) {
  extern __shared__ __align__(16) float sm_raw[];
  float *sm = smem_align128(sm_raw);
  __shared__ long long s_item;
  __shared__ int s_job, s_stop;
  const int tid = threadIdx.x;
  // thread 0's state: the job of its last item (a CTA's items only grow, so
  // the next job is found by a short forward scan) and the last job whose
  // dependencies it saw complete (completion is never undone)
  int last_job = 0, ready_job = -1;
  unsigned long long t_take = 0, t_found = 0, t_ready = 0;
  for (;;) {
    if (tid == 0) {
      s_stop = 0;
      if (stats) t_take = globaltimer_ns();
      const int st0 = ld_relaxed(status);
      const long long it = (long long)atomicAdd(head, 1ull);
      s_item = it;
      if (it >= n_items || st0 != 0) {
        s_stop = 1;
      } else {
        int lo = last_job;
        for (int k = 0; k < 8 && lo + 1 < n_jobs && jobs[lo + 1].first <= it; ++k) ++lo;
        if (lo + 1 < n_jobs && jobs[lo + 1].first <= it) {  // far ahead: bisect
          int hi = n_jobs - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].first <= it) lo = mid;
            else hi = mid - 1;
          }
        }
        last_job = lo;
        s_job = lo;
        if (stats) t_found = globaltimer_ns();
        if (lo != ready_job) {
          const QJob &j = jobs[lo];
          const unsigned long long t0 = globaltimer_ns();
          for (int d = 0; d < kQMaxDeps && !s_stop; ++d) {
            const int dj = j.dep[d];
            if (dj < 0) continue;
            const int need = jobs[dj].type == QJOB_GATE ? 1 : jobs[dj].n_items;
            while (ld_acquire(done + dj) < need) {
              if (ld_acquire(status) != 0) {
                s_stop = 1;
                break;
              }
              if ((long long)(globaltimer_ns() - t0) > wait_limit_ns) {
                atomicOr(status, 1);
                s_stop = 1;
                break;
              }
              __nanosleep(256);
            }
          }
          asm volatile("fence.proxy.async;" ::: "memory");
          if (!s_stop) ready_job = lo;
        }
        if (stats) t_ready = globaltimer_ns();
      }
    }
    __syncthreads();
    if (s_stop) break;
    const QJob &j = jobs[s_job];
    const int c = (int)(s_item - j.first);
    const int t1 = min(j.tiles, (c + 1) * j.per);
    for (int t = c * j.per; t < t1; ++t) {
      ps_queue_tile(j, t, err, sm);
      __syncthreads();  // the tile's shared memory is read before the next one writes it
    }
    // release: the barrier above orders every thread's writes before thread
    // 0's fence and count (the pattern of a grid-wide barrier)
    if (tid == 0) {
      __threadfence();
      atomicAdd(done + s_job, 1);
      if (stats) {  // per job type (slot 3: rows of 48 rotations): take + find, wait, run, tiles
        unsigned long long *st = stats + 4 * (j.type == QJOB_ROWS && j.R == 48 ? 3 : j.type);
        const unsigned long long t_end = globaltimer_ns();
        atomicAdd(st + 0, t_found - t_take);
        atomicAdd(st + 1, t_ready - t_found);
        atomicAdd(st + 2, t_end - t_ready);
        atomicAdd(st + 3, (unsigned long long)(t1 - c * j.per));
      }
    }
  }
}

}  // namespace

size_t ps_queue_smem_rows(int R, int cw, int padx) {
  switch (R) {
    case 12: return rows_smem<12>(R, cw, padx) + kSmemAlign;
    case 24: return rows_smem<24>(R, cw, padx) + kSmemAlign;
    case 48: return rows_smem<48>(R, cw, padx) + kSmemAlign;
    default: return rows_smem<0>(R, cw, padx) + kSmemAlign;
  }
}

size_t ps_queue_smem_cols(int pady) { return cols_tma_smem(pady); }

cudaError_t launch_ps_queue(const QJob *jobs, int n_jobs, long long n_items, unsigned long long *head,
                            int *done, int *status, int *err, long long wait_limit_ns, size_t smem,
                            int *ctas_launched, unsigned long long *stats, cudaStream_t s) {
  if (smem > 227 * 1024 || n_jobs < 1) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_ps_queue, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ps_queue, kQThreads, smem);
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)sms * per_sm;
  if (grid > n_items) grid = n_items > 0 ? n_items : 1;
  if (ctas_launched) *ctas_launched = (int)grid;
  k_ps_queue<<<(unsigned)grid, kQThreads, smem, s>>>(jobs, n_jobs, n_items, head, done, status, err,
                                                      wait_limit_ns, stats);
  return cudaGetLastError();
}

namespace {
}  // namespace

cudaError_t launch_shift_tables(const double *shifts, int n_msgs, int R, int H, int W,
                                int16_t *tables, int4 *sdesc, cudaStream_t s) {
  dim3 grid((unsigned)((2 * R * (W + H) + 255) / 256), (unsigned)n_msgs);
  k_shift_tables<<<grid, 256, 0, s>>>(shifts, R, H, W, tables);
  k_shift_desc<<<(n_msgs * 4 * R + 127) / 128, 128, 0, s>>>(tables, n_msgs, R, H, W, sdesc);
  return cudaGetLastError();
}

cudaError_t launch_msg_rows(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int padx,
                            int *err, cudaStream_t s) {
  switch (R) {
    case 12: return launch_rows_t<12>(msgs, n_msgs, R, H, W, padx, err, s);
    case 24: return launch_rows_t<24>(msgs, n_msgs, R, H, W, padx, err, s);
    case 48: return launch_rows_t<48>(msgs, n_msgs, R, H, W, padx, err, s);
    default: return launch_rows_t<0>(msgs, n_msgs, R, H, W, padx, err, s);
  }
}

cudaError_t launch_msg_rows_cw(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int padx,
                               int cw, int *err, cudaStream_t s) {
  if (cw < 1 || ps_queue_smem_rows(R, cw, padx) > 227 * 1024) return cudaErrorInvalidValue;
  switch (R) {
    case 12: return launch_rows_t<12>(msgs, n_msgs, R, H, W, padx, err, s, cw);
    case 24: return launch_rows_t<24>(msgs, n_msgs, R, H, W, padx, err, s, cw);
    case 48: return launch_rows_t<48>(msgs, n_msgs, R, H, W, padx, err, s, cw);
    default: return launch_rows_t<0>(msgs, n_msgs, R, H, W, padx, err, s, cw);
  }
}

cudaError_t launch_tc_toeplitz(const MsgDesc *msgs, int n_msgs, int H, int W, cudaStream_t s) {
  k_tc_toeplitz<<<dim3(256, (unsigned)n_msgs), 256, 0, s>>>(msgs, H, W);
  return cudaGetLastError();
}

cudaError_t launch_tc_epi(const MsgDesc *msgs, int n_msgs, int R, int H, int W, cudaStream_t s) {
  k_tc_epi<<<dim3((unsigned)((W + kTX - 1) / kTX), (unsigned)(R * ((H + kFullBand - 1) / kFullBand)),
                  (unsigned)n_msgs),
             kThreadsCols, 0, s>>>(msgs, R, H, W);
  return cudaGetLastError();
}

cudaError_t launch_msg_full(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int ohmax,
                            int owmax, int kxmax, int kymax, int *err, cudaStream_t s) {
  (void)err;
  if (ohmax < 1 || owmax < 1 || 2 * kymax + 1 > kMaxFullTaps || (int64_t)R * n_msgs > 65535)
    return cudaErrorInvalidValue;
  const size_t gx_smem = ((size_t)align4(2 * kxmax + 1) + owmax + 2 * kxmax) * sizeof(float);
  if (gx_smem > 227 * 1024) return cudaErrorInvalidValue;
  if ((int64_t)W * H >= ((int64_t)1 << 31) - 1) return cudaErrorInvalidValue;  // 1-based index
  const dim3 gout((unsigned)((owmax + 31) / 32), (unsigned)((ohmax + 7) / 8), (unsigned)(R * n_msgs));
  k_full_fwd<<<gout, dim3(32, 8), 0, s>>>(msgs, R, H, W);
  k_full_dclear<<<gout, dim3(32, 8), 0, s>>>(msgs, R);
  k_full_dscatter<<<dim3((unsigned)((W + 31) / 32), (unsigned)((H + 7) / 8), (unsigned)(R * n_msgs)),
                    dim3(32, 8), 0, s>>>(msgs, R, H, W);
  k_full_dgather<<<gout, dim3(32, 8), 0, s>>>(msgs, R, H, W);
  cudaFuncSetAttribute(k_full_gx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gx_smem);
  k_full_gx<<<dim3((unsigned)ohmax, (unsigned)R, (unsigned)n_msgs), 256, gx_smem, s>>>(msgs, R);
  k_full_gy<<<dim3((unsigned)((owmax + 31) / 32), (unsigned)((ohmax + kFullRows - 1) / kFullRows),
                   (unsigned)(R * n_msgs)),
              dim3(32, 8), 0, s>>>(msgs, R);
  k_full_epi<<<dim3((unsigned)((W + kTX - 1) / kTX), (unsigned)(R * ((H + kFullBand - 1) / kFullBand)),
                    (unsigned)n_msgs),
               kThreadsCols, 0, s>>>(msgs, R, H, W);
  return cudaGetLastError();
}

bool make_src_map(CUtensorMap *m, const float *src, int R, int H, int W) {
  if (W % 4 != 0 || ((uintptr_t)src & 15) != 0 || R < 1 || H < 1) return false;
  return tc::make_map_f32_3d(m, src, (uint64_t)W, (uint64_t)H, (uint64_t)R, kTX, kCBand);
}

bool make_e2_map(CUtensorMap *m, const float *e2, int R, int H, int W) {
  if (W % 4 != 0 || ((uintptr_t)e2 & 15) != 0 || R < 1 || H < 1) return false;
  return tc::make_map_f32_3d(m, e2, (uint64_t)W, (uint64_t)H, (uint64_t)R, kCWT, kCBoxRows);
}

cudaError_t launch_msg_cols(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int pady,
                            int *err, cudaStream_t s, bool tma) {
  if (tma) {
    const size_t smem = cols_tma_smem(pady);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    cudaFuncSetAttribute(k_msg_cols_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int nb = (H + kCBand - 1) / kCBand;
    dim3 grid((unsigned)((W + kTX - 1) / kTX), (unsigned)(R * nb), (unsigned)n_msgs);
    k_msg_cols_tma<<<grid, kColThreads, smem, s>>>(msgs, R, H, W, pady, err);
    return cudaGetLastError();
  }
  // Row band: the whole column when it fits, else halved until it does.
  int band = H;
  auto smem_for = [&](int b) {
    return ((size_t)align4((b + 2 + 2 * pady + kNO + kU) * kCW) + (size_t)align4((b + 2) * kCW) +
            ((2 * pady + 1 + kU - 1) / kU) * kU) * sizeof(float);
  };
  // bands of at most ~56 KB: four CTAs per SM hide the staging and epilogue latency
  while (smem_for(band) > 56 * 1024 && band > 32) band = (band + 1) / 2;
  const size_t smem = smem_for(band);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  cudaFuncSetAttribute(k_msg_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int nb = (H + band - 1) / band;
  dim3 grid((unsigned)((W + kTX - 1) / kTX), (unsigned)(R * nb), (unsigned)n_msgs);
  k_msg_cols<<<grid, kThreadsCols, smem, s>>>(msgs, R, H, W, band, pady, err);
  return cudaGetLastError();
}

}  // namespace pa
