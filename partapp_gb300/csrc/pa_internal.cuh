// pa_internal.cuh -- declarations shared by the CUDA kernels and the host
// orchestration of libpartapp_gb300.  Not part of the public C-ABI.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "partapp_gb300.h"

namespace pa {

constexpr float kLogZero = -1e6f;         // libBoostMath/boost_math.h:23
constexpr float kNoClassValue = 0.0f;     // libPartDetect/partdetect.h:45
constexpr float kClipMin = 0.0001f;       // clip_scores_fill default min_val
constexpr int kMaxRot = 64;               // rotation bins a message kernel handles
constexpr int kMaxRootChildren = 16;
constexpr int kLogZBlocks = 152;          // partial sums per map in launch_log_z

// ---------------------------------------------------------------------------
// Order-preserving integer keys for float max/argmax with atomics.
// fkey: signed-int key, a > b  <=>  fkey(a) > fkey(b) for non-NaN floats.
// akey: 64-bit argmax key: high word orders the value (-0 folded onto +0,
// NaN lowest), low word prefers the smaller flat index (first maximum).
// ---------------------------------------------------------------------------
__host__ __device__ inline int fkey(float f) {
  union { float f; int i; } u;
  u.f = f;
  return u.i >= 0 ? u.i : (u.i ^ 0x7FFFFFFF);
}
__host__ __device__ inline float fkey_decode(int k) {
  union { float f; int i; } u;
  u.i = k >= 0 ? k : (k ^ 0x7FFFFFFF);
  return u.f;
}
constexpr int kFkeyNegInf = (int)(0xFF800000u ^ 0x7FFFFFFFu);  // fkey(-inf)

__host__ __device__ inline uint32_t ukey(float f) {
  union { float f; uint32_t u; } v;
  v.f = f;
  if (f != f) return 0u;            // NaN never wins (reference: '>' is false)
  if (v.u == 0x80000000u) v.u = 0;  // -0 == +0
  return (v.u & 0x80000000u) ? ~v.u : (v.u | 0x80000000u);
}
__host__ __device__ inline float ukey_decode(uint32_t k) {
  union { float f; uint32_t u; } v;
  v.u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return v.f;
}
__host__ __device__ inline unsigned long long akey(float v, uint32_t flat) {
  return ((unsigned long long)ukey(v) << 32) | (unsigned long long)(0xFFFFFFFFu - flat);
}

// ---------------------------------------------------------------------------
// AdaBoost stump table in device memory: {f, p, theta, alpha} per stump,
// plus the per-classifier metadata used by the score-grid kernel.
// ---------------------------------------------------------------------------
struct StumpPart {
  const float4 *stumps;  // .x = f (int bits), .y = p, .z = theta * p, .w = alpha
  const float4 *fast;    // .x = f (int bits), .y = t, .z = p * alpha (p = +-1 only)
  // packed form of `fast` for the 960-dim kernel, npad = n rounded up to 8:
  const uint4 *f8;       // [npad/8] eight uint16 feature indices
  const float4 *ta2;     // [npad/2] {t0, a0, t1, a1}
  int n;
  int npad;
  float sum_alpha;
};

// ---------------------------------------------------------------------------
// SHAPEv5 descriptor grid (k_desc.cu): the per-patch tables and the rotated
// grid of one computeDescriptorGrid call.
// ---------------------------------------------------------------------------
struct DescTables {
  float mask[441];            // initPatchMask(21)
  float lc[441], lr[441];     // (float) precompute_patch_idx, [iradius + j][iradius + i]
  unsigned char inrange[444]; // rx > -1 && rx < 3 && cx > -1 && cx < 4 on the double values
};
struct DescGrid {
  double min_x, min_y, step;            // rect.min_proj_x / min_proj_y, desc_step
  double ax0, ax1, ay0, ay1;            // x_axis, y_axis
  double lo_x, lo_y, hi_x, hi_y;        // inside test and region of interest, intersected
  float v0x, v0y, v1x, v1y;             // patch_scale * axes, as float
  int nx, ny;
  // detection mask [mask_h][mask_w] or null: image position (x, y) reads
  // mask[(long)y - mask_oy][(long)x - mask_ox], 0 outside the array
  const float *mask;
  int mask_w, mask_h, mask_ox, mask_oy;
};
struct IirCoefs {
  float c[17];  // set_smooth_coefficients order (gauss_iir.cpp:77-120)
};
size_t desc_smem_bytes();
// add_image_border2 (libKMA2/ImageContent/ImageContent.cpp:937-999): mirrored border of b pixels
cudaError_t launch_mirror_border(const float *in, int h, int w, int b, float *out, cudaStream_t s);
// squeezeScoreGrid's box (partdetect_test.cpp:407-431): per grid {minx, miny, maxx, maxy} of
// the cells != NO_CLASS_VALUE; grids[g] is [ny][nx]
cudaError_t launch_grid_bbox(const float *const *grids, int n, int ny, int nx, int4 *bbox,
                             cudaStream_t s);
cudaError_t launch_smooth(const float *in, float *tmp, float *out, int h, int w,
                          const IirCoefs &cf, cudaStream_t s);
cudaError_t launch_shape_grid(const float *img, int h, int w, const DescGrid &g,
                              const DescTables *tabs, float *cells, uint8_t *valid,
                              cudaStream_t s);

// ---------------------------------------------------------------------------
// Unary-map descriptor: one (part, rotation) score grid -> log map.
// ---------------------------------------------------------------------------
struct UnaryMap {
  const float *grid;     // [ny][nx]
  float *out;            // [H][W]
  const int *colx;       // separable path: [W] ix1 (TM_BILINEAR) / [nx] ix3 (TM_DIRECT)
  const float *cola;     // [W] bilinear weight a
  const int *rowy;       // [H] iy1 / [ny] iy3
  const float *rowb;     // [H] weight b
  double T13[6];         // general path: grid coords of image pixel (rows 0-1)
  double T31[6];         // general DIRECT path: image coords of grid cell
  int separable;
  int masked_all;        // upright part and this rotation is not kept
  int strip;             // root border strip width in pixels (0 if none)
  int *max_slot;         // fkey of max over the part's masked map
  int ox, oy;            // general DIRECT path: T31 applies to (x1 - ox, y1 - oy)
  // DIRECT maps that may send two cells to one pixel: [H][W] scratch holding
  // the reference's last writer per pixel (null: the map is injective)
  int *order;
};

// ---------------------------------------------------------------------------
// Message descriptor: one computeRotJointMarginal plus the accumulation the
// reference performs with its result.
// ---------------------------------------------------------------------------
enum EpiMode : int {
  EPI_STORE = 0,  // dst0 = m
  EPI_ADD = 1,    // dst0 = m + src0              (post[u] = (0 + m) + unary[u])
  EPI_DOWN = 2,   // dst0 = src0 + m, argmax;      (post[c] += from_root[c])
                  // dst1 = src1 + m, max          (tmp = unary[c] + from_root[c])
};

struct MsgDesc {
  const float *in;        // [R][H][W]
  const CUtensorMap *tm_e2;  // TMA map of e2 as {W, H, R} for the column pass (null: gathered)
  const CUtensorMap *tm_src0, *tm_src1;  // TMA maps of src0 / src1 as {W, H, R} (null: absent)
  const int *in_max;      // fkey of max(in)
  float *e2;              // [R][H][W] row-filtered exp-domain intermediate
  const int16_t *tx_in;   // [R][W] source column in `in` for log_joint_10 column (or -1)
  const int16_t *ty_in;   // [R][H] source row (or -1; all -1 if rotation has no source)
  const int16_t *tx_out;  // [R][W] source column in log_joint_01 for parent column
  const int16_t *ty_out;  // [R][H]
  const int4 *sdesc;      // [4][R] row summaries {c, lo, hi, uniform}: in_x, in_y, out_x, out_y
  const float *rtaps;     // rotation taps (clipped), rlen of them
  const float *xtaps;     // spatial x taps, xlen (odd)
  const float *ytaps;     // spatial y taps, ylen (odd)
  int kidx;               // rot_mean_idx: log_joint_10 rotation = source rotation + kidx
  int rlen;               // -1: rot_sigma == 0 (identity); 0: rot_sigma < 0 (zeros)
  int xlen, ylen;
  int mode;
  float *dst0;
  const float *src0;
  float *dst1;
  const float *src1;
  int *max0;
  int *max1;
  unsigned long long *amax0;
  double *in_max_f64;     // optional FP64 copy of in_M
  // full covariance (gaussFilter2dOffset): the row pass writes the
  // rotation-filtered exp map to e2; it is rotated into the eigenbasis of C
  // (g0 [R][oh][ow]), filtered along the eigen axes (g1, then g0), rotated
  // back bilinearly and logged by the full-covariance epilogue
  int full;
  int oh, ow;
  float *g0, *g1;
  double tf[6];           // rotated-grid cell (x3, y3) -> e2 position (x1, y1)
  double tb[6];           // image cell (x3, y3) -> rotated-grid position
  int sparse;             // bIsSparse: TM_DIRECT forward rotation (e2 cell -> nearest g0 cell)
  double td[6];           // e2 cell (x1, y1) -> rotated-grid position (sparse)
  // tensor-core spatial filter (diagonal C, BF16 operands, FP32 accumulation):
  // the row pass writes the rotation-filtered exp map as bf16 eb [R*H][W]
  // (row stride wp); x pass X^T = Tx * eb^T (xt [W][R*H], bf16), y pass
  // Y_r = Ty * X_r (yv [R][H][W], fp32), then the epilogue
  int tc;
  int wp;                 // row stride of eb (elements, multiple of 8)
  void *eb, *xt;          // bf16
  float *yv;
  void *tbx, *tby;        // bf16 banded Toeplitz matrices [W][W], [H][H] (row strides wp, hp)
  int hp;
};

struct RootDesc {
  const float *msg[kMaxRootChildren];   // root children's messages, joint order
  float *from_root[kMaxRootChildren];
  int *fr_max[kMaxRootChildren];
  int k;
  const float *unary;                   // masked unary of the root
  float *post;                          // post[root] == root marginal
  unsigned long long *amax;
};

// Root of the tree.  In computeRootPosteriorRot (libPictStruct/
// objectdetect_findrot.cpp:630-654) every message from a root child is added
// into post[root] and into log_from_root of every *other* root child, in
// joint order, starting from zero-initialised grids; then the root unary is
// added to post[root], and computePartMarginals (:163-165) adds it to each
// log_from_root.  This performs those sums element-wise in that order on the
// cells first + threadIdx.x + k * stride < N of one block, and folds the
// maxima that the downward messages need and the argmax of the root marginal
// (:261-277) into the descriptor's words (one atomic per block and word).
// KC: the most root children the caller allows (rd.k <= KC); U: cells per
// thread and step, their loads issued together.
template <int KC = kMaxRootChildren, int U = 1>
__device__ __forceinline__ void root_combine_cells(const RootDesc &rd, int64_t first, int64_t N,
                                                   int64_t stride) {
  static_assert(KC <= kMaxRootChildren, "root children");
  const int k = rd.k;
  int keys[KC];
#pragma unroll
  for (int c = 0; c < KC; ++c) keys[c] = kFkeyNegInf;
  unsigned long long am = 0ull;
  // plain loads: inside the persistent queue the messages are written by
  // the same launch
  for (int64_t i0 = first + threadIdx.x; i0 < N; i0 += U * stride) {
    float m[U][KC], u[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int64_t i = i0 + q * stride;
      const bool in = i < N;
#pragma unroll
      for (int c = 0; c < KC; ++c)
        if (c < k) m[q][c] = in ? rd.msg[c][i] : 0.f;
      u[q] = in ? rd.unary[i] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int64_t i = i0 + q * stride;
      if (i >= N) break;
      float s = 0.f;
#pragma unroll
      for (int c = 0; c < KC; ++c)
        if (c < k) s = __fadd_rn(s, m[q][c]);
      const float post = __fadd_rn(s, u[q]);
      rd.post[i] = post;
      const unsigned long long ak = akey(post, (uint32_t)i);
      am = ak > am ? ak : am;
#pragma unroll
      for (int j = 0; j < KC; ++j) {
        if (j >= k) break;
        float fr = 0.f;
#pragma unroll
        for (int c = 0; c < KC; ++c)
          if (c < k && c != j) fr = __fadd_rn(fr, m[q][c]);
        fr = __fadd_rn(fr, u[q]);
        rd.from_root[j][i] = fr;
        keys[j] = max(keys[j], (fr == fr) ? fkey(fr) : kFkeyNegInf);
      }
    }
  }
  __shared__ int skeys[32][kMaxRootChildren];
  __shared__ unsigned long long sam[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int j = 0; j < KC; ++j) {
    const int v = __reduce_max_sync(0xFFFFFFFFu, keys[j]);
    if (lane == 0) skeys[warp][j] = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, am, o);
    am = w > am ? w : am;
  }
  if (lane == 0) sam[warp] = am;
  __syncthreads();
  if ((int)threadIdx.x < k) {
    int v = kFkeyNegInf;
    for (int w = 0; w < nw; ++w) v = max(v, skeys[w][threadIdx.x]);
    atomicMax(rd.fr_max[threadIdx.x], v);
  }
  if (threadIdx.x == 0 && rd.amax) {
    unsigned long long b = 0ull;
    for (int w = 0; w < nw; ++w) b = sam[w] > b ? sam[w] : b;
    atomicMax(rd.amax, b);
  }
  __syncthreads();  // the shared words are read before they are reused
}

// ---------------------------------------------------------------------------
// Persistent message passing (k_ps_queue, k_msg.cu): the row and column
// tiles of every message and the root combinations of many images, drained
// from one device work queue.  A job is a set of independent tiles, taken
// `per` at a time (one queue item); a job may start when each job in `dep`
// has completed all its items.
// ---------------------------------------------------------------------------
enum QJobType { QJOB_ROWS = 0, QJOB_COLS = 1, QJOB_ROOT = 2, QJOB_GATE = 3 };
constexpr int kQMaxDeps = 8;
struct QJob {
  int type;
  int n_items;               // items, ceil(tiles / per) (0 for the gate: the host opens it)
  int tiles;                 // tiles of the job
  int per;                   // tiles per item
  int dep[kQMaxDeps];        // job indices, -1: none
  const MsgDesc *md;         // rows / cols
  const RootDesc *rd;        // root
  int R, H, W;
  int pad;                   // rows: padx of the tile layout; cols: pady
  int cw;                    // rows: column chunk width
  int nch;                   // rows: column chunks per image row; cols: strips
  long long cells;           // root: N; its tiles cover kQRootCells cells each
  long long first;           // queue index of the job's first item
};
constexpr int kQRootCells = 384 * 64;
constexpr int kColBandRows = 176;  // rows of one column-pass tile (kTX columns x one rotation)
constexpr int kColTileCols = 32;
// The row pass with a given column chunk width (the queue's autotuner).
cudaError_t launch_msg_rows_cw(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int padx,
                               int cw, int *err, cudaStream_t s);
constexpr int kQThreads = 384;
// status bits of k_ps_queue: 1 = a dependency wait ran out (the queue was
// abandoned).  stats (optional, [4][4] words: rows, cols, root, rows of 48
// rotations): nanoseconds spent taking and finding items, waiting for
// dependencies, running tiles, and the tile count.
size_t ps_queue_smem_rows(int R, int cw, int padx);
size_t ps_queue_smem_cols(int pady);
cudaError_t launch_ps_queue(const QJob *jobs, int n_jobs, long long n_items, unsigned long long *head,
                            int *done, int *status, int *err, long long wait_limit_ns, size_t smem,
                            int *ctas_launched, unsigned long long *stats, cudaStream_t s);

// Host-side parameters of one computeRotJointMarginal(child -> parent,
// offset_c_10 = oc, offset_p_01 = op, rot_mean, rot_sigma): rotation-mean bin
// shift, clipped rotation taps, spatial taps and the per-rotation shift
// amounts in the reference's double-precision rounding (pa_api.cu).
struct MsgParams {
  int kidx = 0, rlen = -1, xlen = 1, ylen = 1;
  std::vector<float> rtaps, xtaps, ytaps;
  std::vector<double> shifts;  // [4][R]: a_x_in, a_y_in, a_x_out, a_y_out
  bool full = false;           // non-diagonal covariance: taps along the eigen axes
  bool sparse = false;         // bIsSparse: TM_DIRECT forward rotation of a full covariance
  int oh = 0, ow = 0;          // rotated-grid size (transform_grid_resize)
  double tf[6] = {0, 0, 0, 0, 0, 0}, tb[6] = {0, 0, 0, 0, 0, 0}, td[6] = {0, 0, 0, 0, 0, 0};
};
void msg_params(const pa_exp_param *e, double scale, const double *oc, const double *op,
                const double *C, double rot_mean, double rot_sigma, int H, int W, bool sparse,
                MsgParams &m);

// Kernel launchers (defined in the .cu files).  All return cudaGetLastError().
// fast_ok[p] / n_stumps[p] are host arrays describing the classifiers.
// Score grids read field f at fields[f] (a device array) when given, else at
// desc + f * n_loc * dim; fields_aligned: every field pointer is 16-byte
// aligned.
// Rank form of the stump test (k_stump.cu): device tables of one classifier
// set with unit polarities, at most 127 distinct thresholds per feature.
struct RankTables {
  const float *eyt;        // [dim][2^d + 1] per feature: the thresholds in
                           // Eytzinger order at 1 .. 2^d - 1, +inf padded
  const uint2 *rec;        // [n_cls][npad] {f * 128 | (0x80 + k) << 24, bits of -a}
  const float *sum_alpha;  // [n_cls]
  int d, dim, n_cls, npad;
};
size_t rank_bytes(int dim, int64_t n_loc, int n_fields);  // rank tiles of a call
size_t rank_votes_smem(int dim, int n_cls, int npad);
// k_rank_buckets: the rank tiles of the call's descriptors
// (aligned: every field starts on a 16-byte boundary)
cudaError_t launch_rank_buckets(const RankTables &rt, const float *desc,
                                const float *const *fields, bool aligned, int64_t n_loc,
                                int n_fields, uint32_t *ranks, cudaStream_t s);
// k_rank_votes: the score grids from the rank tiles; err bit 8: a tile copy
// did not complete
cudaError_t launch_rank_votes(const RankTables &rt, int64_t n_loc, int n_fields, int normalize,
                              float *scores, const uint32_t *ranks, int *err, cudaStream_t s);
cudaError_t launch_score_grids(const StumpPart *parts_dev, const bool *fast_ok,
                               const int *n_stumps, int n_parts, const float *desc,
                               const float *const *fields, bool fields_aligned,
                               int64_t n_loc_per_field, int n_fields, int dim, int normalize,
                               float *scores, cudaStream_t s);
cudaError_t launch_window_gather(const float *cells, const uint8_t *valid, int n_fields, int ny,
                                 int nx, int dc, int gx, int gy, double grid_step, float *dense,
                                 uint8_t *ok, cudaStream_t s);
cudaError_t launch_mask_no_class(float *scores, const uint8_t *ok, int n_parts, int64_t n_per_part,
                                 cudaStream_t s);
// separable != 0 promises every map uses the column/row tables and that a
// band of 16 image rows reads at most 18 grid rows (|Tig y scale| >= 1).
// ordered: some direct map carries an `order` scratch (a third, gather pass)
cudaError_t launch_unary_maps(const UnaryMap *maps, int n_maps, int ny, int nx, int H, int W,
                              int direct, int separable, int ordered, cudaStream_t s);
cudaError_t launch_prepare_unary(const float *in, float *out, const int *masked_rot, int strip,
                                 int R, int H, int W, int *max_slot, cudaStream_t s);
cudaError_t launch_shift_tables(const double *shifts, int n_msgs, int R, int H, int W,
                                int16_t *tables, int4 *sdesc, cudaStream_t s);
cudaError_t launch_msg_rows(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int padx,
                            int *err_flag, cudaStream_t s);
// BF16 GEMM on tcgen05: C[M][N] (fp32) = A[M][K] * B[N][K]^T, bf16 operands
// with K contiguous (lda, ldb in elements, 16-byte aligned rows).
struct GemmArgs {
  void *C;          // fp32 or bf16 output
  int M, N, K;      // K: the reduction length (columns of A and of B per batch)
  int64_t ldc;      // output row stride (elements)
  int64_t c_batch;  // output offset per batch (elements)
  int b_kofs;       // K offset of B per batch (elements, multiple of 8)
  int band;         // < 0: full K; else the half-width of a banded A
  int out_bf16;
  int vec_ok;       // set by the launcher
};
// A: a_rows x a_cols elements (row stride lda), B: b_rows x b_cols (stride
// ldb); reads outside these extents are zeros; batch = grid.z.
cudaError_t launch_tc_gemm(const void *A, int64_t lda, int64_t a_rows, int64_t a_cols,
                           const void *B, int64_t ldb, int64_t b_rows, int64_t b_cols,
                           const GemmArgs &g, int batch, int *err, cudaStream_t s);
cudaError_t launch_tc_gemm_bf16(const void *A, int64_t lda, const void *B, int64_t ldb, float *C,
                                int64_t ldc, int M, int N, int K, int *err, cudaStream_t s);

// Tensor-core messages of a batch (entries with tc == 0 are skipped): the
// Toeplitz matrices, then the epilogue after the caller's GEMMs.
cudaError_t launch_tc_toeplitz(const MsgDesc *msgs, int n_msgs, int H, int W, cudaStream_t s);
cudaError_t launch_tc_epi(const MsgDesc *msgs, int n_msgs, int R, int H, int W, cudaStream_t s);

// Full-covariance messages of a batch (entries with full == 0 are skipped):
// forward rotation, eigen-axis x and y passes, rotate-back epilogue.
cudaError_t launch_msg_full(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int ohmax,
                            int owmax, int kxmax, int kymax, int *err, cudaStream_t s);
cudaError_t launch_msg_cols(const MsgDesc *msgs, int n_msgs, int R, int H, int W, int pady,
                            int *err_flag, cudaStream_t s, bool tma = false);
// Column-pass TMA map of an e2 buffer [R][H][W] (W a multiple of 4, 16-byte
// aligned); false if it cannot be made.
bool make_e2_map(CUtensorMap *m, const float *e2, int R, int H, int W);
// Column-pass TMA map of an epilogue input (src0 / src1) [R][H][W].
bool make_src_map(CUtensorMap *m, const float *src, int R, int H, int W);
// max_k: the most root children among the descriptors (rd.k <= max_k)
cudaError_t launch_root_combine(const RootDesc *rd, int n_roots, int64_t N, int max_k,
                                cudaStream_t s);
cudaError_t launch_root_posterior(const float *const *post_root, float *const *root_post,
                                  const int *keep, int n_keep, int n_images, int R, int H, int W,
                                  cudaStream_t s);
cudaError_t launch_fill_int(int *p, int v, int64_t n, cudaStream_t s);
// src and dst 16-byte aligned; src may be pinned host memory.
cudaError_t launch_copy16(const void *src, void *dst, int64_t n_words, cudaStream_t s);
cudaError_t launch_map_max(const float *x, int64_t N, int *max_slot, cudaStream_t s);
// findLocalMax of n_maps [S][H][W] grids: up to k (1..2048) maxima per map as
// (s, x, y, value) rows in hyps[map][k][4], their number in n_hyps[map].
size_t local_max_scratch_bytes(int n_maps, int64_t cells, int k);
// findLocalMax in three stages that run in this order on one stream:
// candidates (with the scratch's counters reset), the radix selection, the
// final gather and sort; `stages` is a mask of them.
enum { LM_CAND = 1, LM_SELECT = 2, LM_FINAL = 4, LM_ALL = 7 };
int local_max_kernels(int64_t cells, int k, int stages = LM_ALL);
cudaError_t launch_local_max(const float *const *maps, int n_maps, int S, int H, int W, int k,
                             void *scratch, float *hyps, int *n_hyps, cudaStream_t s,
                             int *n_kernels, int stages = LM_ALL);
cudaError_t launch_argmax(const float *const *maps, int n_maps, int64_t N,
                          unsigned long long *amax, cudaStream_t s);
// log Z of each map in double (float-float partial sums, FP64 total);
// scratch holds log_z_scratch_bytes(n_maps) bytes, 16-byte aligned.
size_t log_z_scratch_bytes(int n_maps);
cudaError_t launch_log_z(const float *const *maps, const unsigned long long *amax, int n_maps,
                         int64_t N, void *scratch, double *log_z, cudaStream_t s);

// Poselet-conditioned extra unaries (k_unary.cu): the rotation score table is
// built on the host, the position and torso terms per pixel on the device.
struct ExtraUnary {
  int root;
  int rot_on, pos_on, torso_on;
  float rot_weight, pos_weight, torso_weight;
  const float *rot_tab;    // [P][R] log rotation scores (float, as the reference stores them)
  const float4 *pos;       // [P] {mu_x, mu_y, var_x, var_y}
  double root_det_x, root_det_y;
  float4 torso;            // {mu_x, mu_y, var_x, var_y}
  float img_cx, img_cy;    // 0.5 * width, 0.5 * height
  const int *is_detect;    // [P] or null (every part detected)
};
cudaError_t launch_extra_unary(const ExtraUnary &ex, float *lu, int P, int S, int R, int H, int W,
                               cudaStream_t s);

// DPM score terms (pa_add_dpm_scores): raw grids [H][W] (torso, head) and
// [P][Rd][H][W] (unary, Rd = R or 1), all >= 0 as the reference loads them.
struct DpmTerms {
  int root, head_part, unary_rot;
  float torso_weight, head_weight, unary_weight;
  const float *torso, *head, *unary;  // null: term off
  double log_floor;                   // log(1e-4) in double
  const int *is_detect;               // [P] or null (every part detected)
  int *err;                           // bit 1: a torso score < 0 or NaN (log undefined)
};
cudaError_t launch_dpm_score(const DpmTerms &dt, float *lu, int P, int S, int R, int H, int W,
                             cudaStream_t s);
// libNms's rectangle form of nms_recursive: rects [n][4][2] corners, scores
// descending; thr = ellipse_size^2 (err bit 1: scores out of order).
cudaError_t launch_nms_rects(const double *rects, const double *score, int n, double thr, int *out,
                             int *err, cudaStream_t s);
cudaError_t launch_nms(const float *x, const float *y, const float *scale, const float *score, int n,
                       double train_w, double train_h, int *out, int *err, cudaStream_t s);

// ---------------------------------------------------------------------------
// Learned unary: convolutions on the tensor cores (k_conv.cu).
// Activations NHWC bf16 [field][row][column][channel]; weights bf16
// [64 out channels][taps * cin] (rows past the layer's outputs zero).
// ---------------------------------------------------------------------------
enum { kConvReluBf16 = 0, kConvOutF32 = 1, kConvMaskBf16 = 2 };
struct ConvArgs {
  int n, H, W, cin_blocks, taps;  // set by launch_conv
  int mode;                       // kConv*
  const float *bias;              // kConvReluBf16 / kConvOutF32: [64] / [n_out]
  void *out;                      // bf16 [pos][64] or fp32 (strided, below)
  const __nv_bfloat16 *act;       // kConvMaskBf16: gradient kept where act > 0
  int n_out;                      // kConvOutF32: channels written (1..64)
  int64_t out_sf, out_sc;         // kConvOutF32: element strides of a field / channel
  int exp_out;                    // kConvOutF32: write exp of the value
  int flat;                       // set by launch_conv: 1x1 over flattened positions
};
struct WgradArgs {
  int H, cin_blocks, taps, n_atoms, m_tiles, xb, kblocks, kb_per_split;
  float *part;  // [splits][m_tiles * 128][64]
};
struct LossArgs {
  const float *pred, *scores;  // fp32, spatial row-major inside a (field, channel) map
  int64_t pred_sf, pred_sc, score_sf, score_sc;
  int n, P, H, W;
  float inv_count;
};
struct AdamArgs {
  float lr, b1, b2, eps, bc1, bc2;
};
struct PackArgs {
  int dim, P;
  int64_t off_w[5];
  __nv_bfloat16 *wf0;    // [64][dim]
  __nv_bfloat16 *wf[4];  // 3x3 layers 1..4, forward [64][9*64]
  __nv_bfloat16 *wd[4];  // 3x3 layers 1..4, input gradient [64][9*64]
};
// conv over `in` (NHWC, cin channels) with `wts`; see ConvArgs for the output.
cudaError_t launch_conv(const void *in, int cin, int taps, int n, int H, int W, const void *wts,
                        const ConvArgs &a, int *err, cudaStream_t s);
size_t conv_wgrad_part_floats(int cin, int taps, int n, int H, int W);
// grad[co][tap][ci] (co < cout) from the layer input `in` and dZ [pos][64].
cudaError_t launch_conv_wgrad(const void *in, int cin, int taps, const void *dz, int n, int H,
                              int W, int cout, float *part, size_t part_floats, float *grad,
                              int *err, cudaStream_t s);
cudaError_t launch_bias_grad(const void *dz, int64_t n_pos, int cout, float *part, int part_blocks,
                             float *grad, cudaStream_t s);
int loss_blocks(int64_t n_pos);
cudaError_t launch_loss_grad(const LossArgs &l, void *dz, float *loss_part, double *loss,
                             cudaStream_t s);
cudaError_t launch_adam(float *p, const float *g, float *m, float *v, int64_t n, const AdamArgs &a,
                        cudaStream_t s);
cudaError_t launch_pack_weights(const float *params, const PackArgs &a, cudaStream_t s);
cudaError_t launch_cast_bf16(const float *src, void *dst, int64_t n, cudaStream_t s);

}  // namespace pa
