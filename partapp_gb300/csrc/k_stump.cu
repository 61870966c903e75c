// k_stump.cu -- dense AdaBoost part detection on GB300.
//
// Replaces the per-location loop of computeScoreGrid
// (libPartDetect/partdetect_test.cpp:366-377) and
// AdaBoostClassifier::evaluateFeaturePoint (libAdaBoost/AdaBoost.h:131-160):
//   s = sum_i ((v[f_i] * p_i < theta_i * p_i) ? alpha_i : -alpha_i);  s /= sum_alpha
// Each thread owns one (location, part) pair and walks the part's stumps in
// the reference's order, so every decision and the float sum are bit-exact.
//
// Layout: a CTA stages kLoc = 32 consecutive locations of one field in shared
// memory (row = one location's dim-long vector).  Element f of location l is
// stored at l * dp + (f ^ l): the XOR swizzle spreads the 32 lanes of a warp
// (32 locations reading the same feature f) over 32 banks.  Warp w evaluates
// part w of the CTA's part group, lane l evaluates location l, so the stump
// record a warp reads is uniform (broadcast load).
#include "pa_internal.cuh"
#include "tc_common.cuh"

namespace pa {
namespace {

constexpr int kLoc = 32;

__global__ void __launch_bounds__(512) k_score_grids(const StumpPart *__restrict__ parts,
                                                     int n_parts, const float *__restrict__ desc,
                                                     const float *const *__restrict__ fields,
                                                     int64_t n_loc, int dim, int dp,
                                                     int normalize, float *__restrict__ scores,
                                                     int n_fields) {
  extern __shared__ float sm[];
  const int field = blockIdx.y;
  const int64_t loc0 = (int64_t)blockIdx.x * kLoc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const float *src = (fields ? fields[field] : desc + (int64_t)field * n_loc * dim) + loc0 * dim;
  const int nl = (n_loc - loc0) < kLoc ? (int)(n_loc - loc0) : kLoc;

  // Stage the tile: warp-contiguous global reads, swizzled conflict-free stores.
  for (int l = warp; l < kLoc; l += nwarps) {
    float *row = sm + l * dp;
    if (l < nl) {
      const float *g = src + (int64_t)l * dim;
      for (int c = lane; c < dim; c += 32) row[c ^ l] = __ldg(g + c);
    } else {
      for (int c = lane; c < dp; c += 32) row[c] = 0.f;
    }
  }
  __syncthreads();

  const int part = blockIdx.z * nwarps + warp;
  if (part >= n_parts || lane >= nl) return;
  const StumpPart sp = parts[part];
  const float4 *__restrict__ st = sp.stumps;
  const float *v = sm + lane * dp;
  float s = 0.f;
#pragma unroll 4
  for (int i = 0; i < sp.n; ++i) {
    const float4 q = __ldg(st + i);
    const float val = v[__float_as_int(q.x) ^ lane];
    s += (__fmul_rn(val, q.y) < q.z) ? q.w : -q.w;
  }
  if (normalize) s = __fdiv_rn(s, sp.sum_alpha);
  scores[((int64_t)part * n_fields + field) * n_loc + loc0 + lane] = s;
}

// FeatureGrid::concatenate (libPartDetect/FeatureGrid.cpp:137-181): window
// vector of (ix, iy) = reverse-order concatenation of the gx*gy cells at
// (ix + round(kx*grid_step), iy + round(ky*grid_step)); ok = 0 past
// last_valid_grid_pos (FeatureGrid.h:71-75) or when a cell is missing.
__global__ void k_window_gather(const float *__restrict__ cells, const uint8_t *__restrict__ valid,
                                int ny, int nx, int dc, int gx, int gy, double grid_step,
                                int last_ix, int last_iy, float *__restrict__ dense,
                                uint8_t *__restrict__ ok) {
  const int field = blockIdx.z;
  const int iy = blockIdx.y;
  const int D = gx * gy * dc;
  for (int ix = blockIdx.x; ix < nx; ix += gridDim.x) {
    const int64_t loc = ((int64_t)field * ny + iy) * nx + ix;
    float *out = dense + loc * D;
    bool good = (ix <= last_ix && iy <= last_iy);
    if (good) {
      for (int k = 0; k < gx * gy; ++k) {
        const int ky = k / gx, kx = k - ky * gx;
        const int x = ix + (int)floor(kx * grid_step + 0.5);
        const int y = iy + (int)floor(ky * grid_step + 0.5);
        if (!valid[((int64_t)field * ny + y) * nx + x]) good = false;
      }
    }
    if (threadIdx.x == 0) ok[loc] = good ? 1 : 0;
    if (!good) {
      for (int c = threadIdx.x; c < D; c += blockDim.x) out[c] = 0.f;
      continue;
    }
    for (int k = 0; k < gx * gy; ++k) {
      const int ky = k / gx, kx = k - ky * gx;
      const int x = ix + (int)floor(kx * grid_step + 0.5);
      const int y = iy + (int)floor(ky * grid_step + 0.5);
      const float *cell = cells + (((int64_t)field * ny + y) * nx + x) * dc;
      float *dstc = out + (int64_t)(gx * gy - 1 - k) * dc;
      for (int c = threadIdx.x; c < dc; c += blockDim.x) dstc[c] = cell[c];
    }
  }
}

// The same gather with 16-byte copies, one warp per window (dc % 4 == 0 and
// 16-byte aligned cells and windows): the window's cells are copied by all
// lanes at once; the cell offsets round(k * grid_step) come from a table.
struct CellOffsets {
  int2 o[64];  // (round(kx * grid_step), round(ky * grid_step)) for k = ky * gx + kx
};

__global__ void __launch_bounds__(256) k_window_gather4(
    const float4 *__restrict__ cells, const uint8_t *__restrict__ valid, int n_fields, int ny,
    int nx, int dc4, int gx, int gy, const CellOffsets offs_t, int last_ix, int last_iy,
    float4 *__restrict__ dense, uint8_t *__restrict__ ok) {
  const int2 *offs = offs_t.o;
  const int lane = threadIdx.x & 31;
  const int K = gx * gy, D4 = K * dc4;
  const int64_t n_win = (int64_t)n_fields * ny * nx;
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t win = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); win < n_win;
       win += wstride) {
    const int field = (int)(win / ((int64_t)ny * nx));
    const int rem = (int)(win - (int64_t)field * ny * nx);
    const int iy = rem / nx, ix = rem - (rem / nx) * nx;
    bool good = ix <= last_ix && iy <= last_iy;
    if (good) {
      bool mine = true;
      for (int k = lane; k < K; k += 32)
        mine = mine && valid[((int64_t)field * ny + iy + offs[k].y) * nx + ix + offs[k].x] != 0;
      good = __all_sync(0xFFFFFFFFu, mine);
    }
    float4 *out = dense + win * D4;
    if (lane == 0) ok[win] = good ? 1 : 0;
    if (!good) {
      for (int j = lane; j < D4; j += 32) out[j] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    for (int j = lane; j < D4; j += 32) {
      const int k = j / dc4, o = j - (j / dc4) * dc4;
      const float4 *cell =
          cells + (((int64_t)field * ny + iy + offs[k].y) * nx + ix + offs[k].x) * dc4;
      out[(int64_t)(K - 1 - k) * dc4 + o] = __ldg(cell + o);
    }
  }
}

__global__ void k_mask_no_class(float *__restrict__ scores, const uint8_t *__restrict__ ok,
                                int64_t n_per_part, int n_parts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_per_part) return;
  if (!ok[i])
    for (int p = 0; p < n_parts; ++p) scores[(int64_t)p * n_per_part + i] = kNoClassValue;
}

// ---------------------------------------------------------------------------
// Pipelined variant for 960-dim descriptors.
//
// The classifiers are split into G groups of at most kMaxWarps; a CTA serves
// one group and keeps that group's stump tables resident in shared memory
// for the whole launch.  The CTAs of the G groups walk the tiles in the same
// order, so the second read of a tile is an L2 hit.
//
// Persistent CTAs walk the tiles; while a tile is being evaluated, the next
// tile is already in flight into registers (kChunks float4 per thread).
// Rows are stored with a stride of DIM + 1 floats, so the 32 lanes (32
// locations) reading one feature hit 32 banks, and a warp's staging store of
// 4 rows x 8 float4 chunks hits bank (l + 4q + j) mod 32, again all 32 banks.
//
// Stump records are {f, t, a, -}: for a polarity p = +1 the test
// v*p < theta*p is v < theta; for p = -1 it is v > theta, i.e.
// !(v < nextafter(theta, +inf)).  With t = theta or nextafter(theta, +inf)
// and a = p*alpha the reference's vote (v*p < theta*p) ? alpha : -alpha is
// (v < t) ? a : -a for every non-NaN v -- one compare, one select, one add.
// Classifiers with other polarities use the literal form (k_score_grids).
// ---------------------------------------------------------------------------
constexpr int kChunks = 24;
constexpr int kMaxWarps = 11;

template <int DIM>
__global__ void __launch_bounds__(32 * kMaxWarps, 1) k_score_grids_pipe(
    const StumpPart *__restrict__ parts, int n_parts, int n_groups, int group_size,
    const float *__restrict__ desc, const float *const *__restrict__ fields, int64_t n_loc,
    int normalize, float *__restrict__ scores,
    int n_fields) {
  static_assert(DIM % 32 == 0, "DIM must be a multiple of 32");
  constexpr int kCpr = DIM / 4;          // float4 chunks per row
  constexpr int kBlk = 8 * (kCpr / 8);   // 4-row x 8-chunk blocks per tile
  constexpr int kStride = DIM + 1;       // padded shared-memory row
  extern __shared__ __align__(16) float sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int group = blockIdx.x % n_groups;
  const int cta_in_group = blockIdx.x / n_groups;
  const int ctas_per_group = gridDim.x / n_groups;
  // this warp's classifier (warps past the group size only stage tiles)
  const int part = warp < group_size ? group * group_size + warp : n_parts;
  const int64_t blocks_per_field = (n_loc + kLoc - 1) / kLoc;
  const int64_t n_tiles = blocks_per_field * n_fields;
  const int lrow = lane >> 3, lchunk = lane & 7;

  // resident packed stump tables of the group: per classifier
  // f8[npad/8] (uint4) followed by ta2[npad/2] (float4)
  char *stab = reinterpret_cast<char *>(sm + 32 * kStride);
  int my_npad = 0;
  float my_sum_alpha = 1.f;
  const uint4 *my_f8 = nullptr;
  const float4 *my_ta = nullptr;
  {
    size_t off = 0;
    for (int w = 0; w < group_size && w < nwarps; ++w) {
      const int pw = group * group_size + w;
      if (pw >= n_parts) break;
      const StumpPart sp = parts[pw];
      uint4 *f8 = reinterpret_cast<uint4 *>(stab + off);
      float4 *ta = reinterpret_cast<float4 *>(stab + off + (size_t)sp.npad * 2);
      if (w == warp) {
        my_npad = sp.npad;
        my_sum_alpha = sp.sum_alpha;
        my_f8 = f8;
        my_ta = ta;
        for (int i = lane; i < sp.npad / 8; i += 32) f8[i] = __ldg(sp.f8 + i);
        for (int i = lane; i < sp.npad / 2; i += 32) ta[i] = __ldg(sp.ta2 + i);
      }
      off += (size_t)sp.npad * 10;
    }
  }

  float4 st[kChunks];
  auto load_tile = [&](int64_t tt) {
    const int field = (int)(tt / blocks_per_field);
    const int64_t loc0 = (tt - (int64_t)field * blocks_per_field) * kLoc;
    const int nl = (n_loc - loc0) < kLoc ? (int)(n_loc - loc0) : kLoc;
    const float *fb = fields ? fields[field] : desc + (int64_t)field * n_loc * DIM;
    const float4 *src = reinterpret_cast<const float4 *>(fb + loc0 * DIM) +
                        lrow * kCpr + 24 * warp + lchunk;
#pragma unroll
    for (int k = 0; k < kChunks; ++k) {
      const int g = warp * kChunks + k;
      const int l = 4 * (k & 7) + lrow;
      if (g < kBlk && l < nl) st[k] = __ldg(src + (4 * (k & 7)) * kCpr + 8 * (k >> 3));
      else st[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };

  int64_t t = cta_in_group;
  if (t < n_tiles) load_tile(t);
  for (; t < n_tiles; t += ctas_per_group) {
    __syncthreads();  // the previous tile is no longer read (first pass: stump tables staged)
#pragma unroll
    for (int k = 0; k < kChunks; ++k) {
      const int g = warp * kChunks + k;
      if (g < kBlk) {
        const int l = 4 * (k & 7) + lrow;
        float *dst = sm + l * kStride + 4 * (8 * (3 * warp + (k >> 3)) + lchunk);
        dst[0] = st[k].x;
        dst[1] = st[k].y;
        dst[2] = st[k].z;
        dst[3] = st[k].w;
      }
    }
    __syncthreads();
    if (t + ctas_per_group < n_tiles) load_tile(t + ctas_per_group);
    if (part < n_parts) {
      const int field = (int)(t / blocks_per_field);
      const int64_t loc0 = (t - (int64_t)field * blocks_per_field) * kLoc;
      const int nl = (n_loc - loc0) < kLoc ? (int)(n_loc - loc0) : kLoc;
      const float *v = sm + lane * kStride;
      float s = 0.f;
#pragma unroll 4
      for (int j = 0; j < my_npad / 8; ++j) {
        const uint4 fq = my_f8[j];
        const float4 q0 = my_ta[4 * j], q1 = my_ta[4 * j + 1];
        const float4 q2 = my_ta[4 * j + 2], q3 = my_ta[4 * j + 3];
        s += (v[fq.x & 0xFFFFu] < q0.x) ? q0.y : -q0.y;
        s += (v[fq.x >> 16] < q0.z) ? q0.w : -q0.w;
        s += (v[fq.y & 0xFFFFu] < q1.x) ? q1.y : -q1.y;
        s += (v[fq.y >> 16] < q1.z) ? q1.w : -q1.w;
        s += (v[fq.z & 0xFFFFu] < q2.x) ? q2.y : -q2.y;
        s += (v[fq.z >> 16] < q2.z) ? q2.w : -q2.w;
        s += (v[fq.w & 0xFFFFu] < q3.x) ? q3.y : -q3.y;
        s += (v[fq.w >> 16] < q3.z) ? q3.w : -q3.w;
      }
      if (normalize) s = __fdiv_rn(s, my_sum_alpha);
      if (lane < nl) scores[((int64_t)part * n_fields + field) * n_loc + loc0 + lane] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Rank form of the stump test (classifier sets with unit polarities).
//
// For a feature f let U_f = {u_0 < u_1 < ... < u_{m-1}} be the distinct
// thresholds t (of the sign-folded records above) that the set's stumps put
// on f.  The rank of a value v is b(v) = #{u in U_f : u <= v} (a NaN ranks
// above every threshold).  A stump (f, t = u_k) has v < t exactly when
// b(v) <= k, so with m <= 127 every test is a byte comparison:
//
// k_rank_buckets: every descriptor value -> its rank byte by a d-step search
//   of the feature's thresholds, stored in Eytzinger order (shared memory).
//   Output: tiles of kRankLoc = 128 locations of one field, word (f, g) of a
//   tile = the ranks of locations 4g .. 4g+3 (byte j = location 4g + j).
// k_rank_votes: one warp per classifier walks its stumps in order over a
//   tile bulk-copied into shared memory.  One 32-bit load gives lane g the
//   ranks of four locations and one subtraction tests all four:
//     d = (0x80 + k) * 0x01010101 - ranks,  bit 7 of byte j set <=> b_j <= k
//   (0x80 + k - b lies in [1, 254]: no borrow crosses a byte; the record
//   keeps 0x80 + k in its top byte, replicated by one byte permute).  The
//   vote is -a with its sign bit flipped when the test holds.  Each
//   location's votes are summed in stump order, as in the float kernels, so
//   the scores are the same bits.  Padding records (k = 127, -a = -0) vote
//   +0.
// NaN descriptor values rank above every threshold: their test is false, as
// v < t is.
// ---------------------------------------------------------------------------
constexpr int kRankLoc = 128;       // locations per tile
constexpr int kRankSlab = 8;        // feature groups of 32 per k_rank_buckets CTA
constexpr int kRankWarps1 = 16;     // k_rank_buckets
constexpr int kRankMaxWarps = 32;   // k_rank_votes: one warp per classifier

// A CTA serves one slab of 256 features (kRankSlab groups of 32) for a
// strided set of tiles.  Lane g of a warp reads the slab of one location as
// two float4 (features 128c + 4g .. 128c + 4g + 3, c = 0, 1): value u = 4c + j
// of lane g is local feature fl(u, g) = 128c + 4g + j.  Shared tables and
// output rows are kept in (u, g) order so that every access is one bank per
// lane: thresholds as [u][entry][g], output rows r = 32u + g (stride 33).
template <int D, bool VEC>
__global__ void __launch_bounds__(32 * kRankWarps1) k_rank_buckets(
    const float *__restrict__ eyt, int dim, const float *__restrict__ desc,
    const float *const *__restrict__ fields, int64_t n_loc, int n_fields,
    uint32_t *__restrict__ ranks) {
  extern __shared__ __align__(16) float sm[];
  constexpr int S = (1 << D) + 1;  // row stride of the global table
  constexpr int T = 1 << D;        // entries per feature in shared memory
  constexpr int SLAB = kRankSlab * 32;
  const int n_slabs = (dim + SLAB - 1) / SLAB;
  const int slab = blockIdx.x % n_slabs;
  const int cta = blockIdx.x / n_slabs, n_cta = gridDim.x / n_slabs;
  const int f0 = slab * SLAB, nf = min(dim, f0 + SLAB) - f0;  // nf: a multiple of 4
  float *tab = sm;                                                     // [8][T][32]
  uint32_t *os = reinterpret_cast<uint32_t *>(sm + (size_t)kRankSlab * T * 32);  // [8 * 32][33]
  unsigned char *osb = reinterpret_cast<unsigned char *>(os);
  for (int i = threadIdx.x; i < kRankSlab * T * 32; i += blockDim.x) {
    const int u = i / (T * 32), e = (i / 32) % T, g = i & 31;
    const int fl = (u >> 2) * 128 + 4 * g + (u & 3);
    tab[i] = fl < nf ? __ldg(eyt + (size_t)(f0 + fl) * S + e) : INFINITY;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t tiles_per_field = (n_loc + kRankLoc - 1) / kRankLoc;
  const int64_t n_tiles = tiles_per_field * n_fields;
  const bool in0 = 4 * lane < nf, in1 = 128 + 4 * lane < nf;
  // one location per warp at a time, the next one's loads in flight while
  // this one is searched
  auto load = [&](const float *p, bool ok, float *v4) {
    if (VEC) {
      const float4 x = ok ? __ldg(reinterpret_cast<const float4 *>(p)) : make_float4(0.f, 0.f, 0.f, 0.f);
      v4[0] = x.x, v4[1] = x.y, v4[2] = x.z, v4[3] = x.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) v4[j] = ok ? __ldg(p + j) : 0.f;
    }
  };
  // slab base of tile t's field and the tile's first location
  auto tile_src = [&](int64_t t, int64_t &loc0) {
    const int field = (int)(t / tiles_per_field);
    loc0 = (t - (int64_t)field * tiles_per_field) * kRankLoc;
    return (fields ? fields[field] : desc + (int64_t)field * n_loc * dim) + f0 + 4 * lane;
  };
  float v[8], vn[8];
  if (cta < n_tiles) {
    int64_t loc0;
    const float *fb = tile_src(cta, loc0);
    const int64_t loc = loc0 + warp;
    load(fb + loc * dim, in0 && loc < n_loc, v);
    load(fb + loc * dim + 128, in1 && loc < n_loc, v + 4);
  }
  for (int64_t t = cta; t < n_tiles; t += n_cta) {
    int64_t loc0, loc0n = 0;
    const float *fb = tile_src(t, loc0);
    // the location after the last one of this tile: the next tile's first
    const float *fbn = t + n_cta < n_tiles ? tile_src(t + n_cta, loc0n) : fb;
    for (int l = warp; l < kRankLoc; l += nw) {
      const bool here = l + nw < kRankLoc;
      const int64_t locn = here ? loc0 + l + nw : loc0n + warp;
      const float *src = here ? fb : fbn;
      const bool more = (here || t + n_cta < n_tiles) && locn < n_loc;
      load(src + locn * dim, in0 && more, vn);
      load(src + locn * dim + 128, in1 && more, vn + 4);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        // step right unless v < entry: "v >= entry or unordered", so a NaN
        // takes the last leaf, rank 2^D - 1, above every threshold index
        const float *col = tab + u * T * 32 + lane;
        int i = 1;
#pragma unroll
        for (int st = 0; st < D; ++st) {
          uint32_t m;
          asm("set.geu.u32.f32 %0, %1, %2;" : "=r"(m) : "f"(v[u]), "f"(col[i * 32]));
          i = 2 * i - (int)m;
        }
        osb[((size_t)(u * 32 + lane) * 33 + (l >> 2)) * 4 + (l & 3)] =
            (unsigned char)(i - (1 << D));
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = vn[u];
    }
    __syncthreads();
    // rows back in feature order: feature fl sits in row 32 * (4c + j) + g
    uint32_t *dst = ranks + ((size_t)t * dim + f0) * 32;
    for (int i = threadIdx.x; i < nf * 32; i += blockDim.x) {
      const int fl = i >> 5;
      const int r = ((fl >> 7) * 4 + (fl & 3)) * 32 + ((fl >> 2) & 31);
      dst[i] = os[r * 33 + (i & 31)];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(32 * kRankMaxWarps, 1) k_rank_votes(
    const uint2 *__restrict__ rec, const float *__restrict__ sum_alpha, int n_cls, int npad,
    int dim, const uint32_t *__restrict__ ranks, int64_t n_loc, int n_fields, int normalize,
    float *__restrict__ scores, int *err) {
  extern __shared__ __align__(16) unsigned char smr[];
  // tile [dim][32] words at the first 128-byte boundary, then the records
  unsigned char *base =
      smr + ((128 - (tc::smem_u32(smr) & 127u)) & 127u);
  uint32_t *tile = reinterpret_cast<uint32_t *>(base);
  uint2 *srec = reinterpret_cast<uint2 *>(base + (size_t)dim * 128);
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_ok;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n_cls * npad; i += blockDim.x) srec[i] = rec[i];
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int64_t tiles_per_field = (n_loc + kRankLoc - 1) / kRankLoc;
  const int64_t n_tiles = tiles_per_field * n_fields;
  const uint32_t tile_bytes = (uint32_t)dim * 128u, chunk = tile_bytes / 4u;  // dim * 32: 16-byte multiple
  uint32_t phase = 0;
  for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x, phase ^= 1u) {
    if (tid == 0) {
      const unsigned char *src = reinterpret_cast<const unsigned char *>(ranks) + (size_t)t * tile_bytes;
      tc::mbar_arrive_expect_tx(&bar, tile_bytes);
      for (int c = 0; c < 4; ++c) tc::bulk_load(base + c * chunk, src + c * chunk, chunk, &bar);
      if (t + gridDim.x < n_tiles) tc::bulk_prefetch_l2(src + (size_t)gridDim.x * tile_bytes, tile_bytes);
      s_ok = tc::mbar_wait_try(&bar, phase, err) ? 1 : 0;
      if (!s_ok) tc::mbar_wait_try(&bar, phase, err);  // once more for the copies in flight
    }
    __syncthreads();
    if (!s_ok) break;
    if (warp < n_cls) {
      const int field = (int)(t / tiles_per_field);
      const int64_t loc0 = (t - (int64_t)field * tiles_per_field) * kRankLoc;
      const uint2 *r = srec + (size_t)warp * npad;
      const unsigned char *lane_base = base + lane * 4;
      // locations 0, 1 and 2, 3 summed in pairs by packed adds (two IEEE
      // float adds each, the same order as scalar sums)
      unsigned long long s01 = 0ull, s23 = 0ull;
#pragma unroll 4
      for (int i = 0; i < npad; ++i) {
        const uint2 q = r[i];
        const uint32_t w = *reinterpret_cast<const uint32_t *>(lane_base + (q.x & 0x1FFFFu));
        const uint32_t d = __byte_perm(q.x, 0u, 0x3333u) - w;
        const uint32_t v0 = q.y ^ ((d << 24) & 0x80000000u), v1 = q.y ^ ((d << 16) & 0x80000000u);
        const uint32_t v2 = q.y ^ ((d << 8) & 0x80000000u), v3 = q.y ^ (d & 0x80000000u);
        const unsigned long long a01 = ((unsigned long long)v1 << 32) | v0;
        const unsigned long long a23 = ((unsigned long long)v3 << 32) | v2;
        asm("add.rn.f32x2 %0, %0, %1;" : "+l"(s01) : "l"(a01));
        asm("add.rn.f32x2 %0, %0, %1;" : "+l"(s23) : "l"(a23));
      }
      float s0 = __uint_as_float((uint32_t)s01), s1 = __uint_as_float((uint32_t)(s01 >> 32));
      float s2 = __uint_as_float((uint32_t)s23), s3 = __uint_as_float((uint32_t)(s23 >> 32));
      if (normalize) {
        const float sa = sum_alpha[warp];
        s0 = __fdiv_rn(s0, sa);
        s1 = __fdiv_rn(s1, sa);
        s2 = __fdiv_rn(s2, sa);
        s3 = __fdiv_rn(s3, sa);
      }
      float *o = scores + ((int64_t)warp * n_fields + field) * n_loc + loc0 + 4 * lane;
      const int64_t left = n_loc - (loc0 + 4 * lane);
      if (left > 0) o[0] = s0;
      if (left > 1) o[1] = s1;
      if (left > 2) o[2] = s2;
      if (left > 3) o[3] = s3;
    }
    __syncthreads();  // the tile is read before the next copy overwrites it
  }
  __syncthreads();
  if (tid == 0) tc::mbar_inval(&bar);
}

}  // namespace

cudaError_t launch_score_grids(const StumpPart *parts_dev, const bool *fast_ok,
                               const int *n_stumps, int n_parts, const float *desc,
                               const float *const *fields, bool fields_aligned,
                               int64_t n_loc, int n_fields, int dim, int normalize,
                               float *scores, cudaStream_t s) {
  // pipelined kernel: groups of <= kMaxWarps classifiers with resident
  // stump tables; needs 960-dim descriptors, unit polarities and room for
  // the tables next to the 32 x 961 tile.
  const bool aligned = fields ? fields_aligned : ((uintptr_t)desc & 15) == 0;
  bool all_fast = true;
  for (int p = 0; p < n_parts; ++p) all_fast = all_fast && fast_ok[p];
  const int n_groups = (n_parts + kMaxWarps - 1) / kMaxWarps;
  const int nw = (n_parts + n_groups - 1) / n_groups;
  size_t max_group_stumps = 0;
  for (int g = 0; g < n_groups; ++g) {
    size_t tot = 0;
    for (int p = g * nw; p < n_parts && p < (g + 1) * nw; ++p) tot += (size_t)n_stumps[p];
    max_group_stumps = tot > max_group_stumps ? tot : max_group_stumps;
  }
  const size_t tile_bytes = ((size_t)kLoc * 961 + 3) / 4 * 4 * sizeof(float);
  const size_t smem_pipe = tile_bytes + max_group_stumps * 10;  // 2 B index + 8 B {t, a}
  const int launch_warps = nw < 10 ? 10 : nw;  // ten warps stage a 960-wide tile
  if (dim == 960 && aligned && all_fast && smem_pipe <= 227 * 1024) {
    cudaFuncSetAttribute(k_score_grids_pipe<960>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem_pipe);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t n_tiles = ((n_loc + kLoc - 1) / kLoc) * n_fields;
    int64_t per_group = sms / n_groups;
    if (per_group < 1) per_group = 1;
    if (per_group > n_tiles) per_group = n_tiles;
    k_score_grids_pipe<960><<<(unsigned)(per_group * n_groups), 32 * launch_warps, smem_pipe, s>>>(
        parts_dev, n_parts, n_groups, nw, desc, fields, n_loc, normalize, scores, n_fields);
    return cudaGetLastError();
  }
  const int dp = (dim + 31) & ~31;
  const size_t smem = (size_t)kLoc * dp * sizeof(float);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_score_grids, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    attr_set = true;
  }
  const int gw = n_parts < 16 ? n_parts : 16;
  dim3 grid((unsigned)((n_loc + kLoc - 1) / kLoc), (unsigned)n_fields,
            (unsigned)((n_parts + gw - 1) / gw));
  k_score_grids<<<grid, 32 * gw, smem, s>>>(parts_dev, n_parts, desc, fields, n_loc, dim, dp, normalize,
                                            scores, n_fields);
  return cudaGetLastError();
}

size_t rank_bytes(int dim, int64_t n_loc, int n_fields) {
  return (size_t)((n_loc + kRankLoc - 1) / kRankLoc) * n_fields * dim * 128;
}

size_t rank_votes_smem(int dim, int n_cls, int npad) {
  return 128 + (size_t)dim * 128 + (size_t)n_cls * npad * sizeof(uint2);
}

cudaError_t launch_rank_buckets(const RankTables &rt, const float *desc,
                                const float *const *fields, bool aligned, int64_t n_loc,
                                int n_fields, uint32_t *ranks, cudaStream_t s) {
  if (rt.d < 1 || rt.d > 7 || rt.n_cls < 1 || rt.n_cls > kRankMaxWarps || rt.dim > 1023 ||
      rt.dim % 4 || rank_votes_smem(rt.dim, rt.n_cls, rt.npad) > 227 * 1024)
    return cudaErrorInvalidValue;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int n_slabs = (rt.dim + kRankSlab * 32 - 1) / (kRankSlab * 32);
  const size_t smem1 = (size_t)kRankSlab * 32 * (((size_t)1 << rt.d) + 33) * sizeof(float);
  const int64_t n_tiles = ((n_loc + kRankLoc - 1) / kRankLoc) * n_fields;
  auto go1 = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
    if (e != cudaSuccess) return e;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kRankWarps1, smem1);
    if (per_sm < 1) per_sm = 1;
    int64_t per_slab = ((int64_t)sms * per_sm + n_slabs - 1) / n_slabs;
    if (per_slab > n_tiles) per_slab = n_tiles;
    kern<<<(unsigned)(per_slab * n_slabs), 32 * kRankWarps1, smem1, s>>>(rt.eyt, rt.dim, desc, fields,
                                                                         n_loc, n_fields, ranks);
    return cudaGetLastError();
  };
  cudaError_t e = cudaSuccess;
  switch (rt.d * 2 + (aligned ? 1 : 0)) {
    case 2: e = go1(k_rank_buckets<1, false>); break;
    case 3: e = go1(k_rank_buckets<1, true>); break;
    case 4: e = go1(k_rank_buckets<2, false>); break;
    case 5: e = go1(k_rank_buckets<2, true>); break;
    case 6: e = go1(k_rank_buckets<3, false>); break;
    case 7: e = go1(k_rank_buckets<3, true>); break;
    case 8: e = go1(k_rank_buckets<4, false>); break;
    case 9: e = go1(k_rank_buckets<4, true>); break;
    case 10: e = go1(k_rank_buckets<5, false>); break;
    case 11: e = go1(k_rank_buckets<5, true>); break;
    case 12: e = go1(k_rank_buckets<6, false>); break;
    case 13: e = go1(k_rank_buckets<6, true>); break;
    case 14: e = go1(k_rank_buckets<7, false>); break;
    default: e = go1(k_rank_buckets<7, true>); break;
  }
  return e;
}

cudaError_t launch_rank_votes(const RankTables &rt, int64_t n_loc, int n_fields, int normalize,
                              float *scores, const uint32_t *ranks, int *err, cudaStream_t s) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t n_tiles = ((n_loc + kRankLoc - 1) / kRankLoc) * n_fields;
  const size_t smem2 = rank_votes_smem(rt.dim, rt.n_cls, rt.npad);
  cudaError_t e;
  e = cudaFuncSetAttribute(k_rank_votes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
  if (e != cudaSuccess) return e;
  const int warps = rt.n_cls < 8 ? 8 : rt.n_cls;
  int64_t grid = sms;
  if (grid > n_tiles) grid = n_tiles;
  k_rank_votes<<<(unsigned)grid, 32 * warps, smem2, s>>>(rt.rec, rt.sum_alpha, rt.n_cls, rt.npad,
                                                         rt.dim, ranks, n_loc, n_fields, normalize,
                                                         scores, err);
  return cudaGetLastError();
}

cudaError_t launch_window_gather(const float *cells, const uint8_t *valid, int n_fields, int ny,
                                 int nx, int dc, int gx, int gy, double grid_step, float *dense,
                                 uint8_t *ok, cudaStream_t s) {
  const int last_ix = nx - (int)floor(grid_step * (gx - 1) + 0.5) - 1;
  const int last_iy = ny - (int)floor(grid_step * (gy - 1) + 0.5) - 1;
  const int K = gx * gy;
  if (dc % 4 == 0 && K <= 64 && ((uintptr_t)cells & 15) == 0 && ((uintptr_t)dense & 15) == 0) {
    CellOffsets t;
    for (int k = 0; k < K; ++k) {
      const int ky = k / gx, kx = k - ky * gx;
      t.o[k] = make_int2((int)floor(kx * grid_step + 0.5), (int)floor(ky * grid_step + 0.5));
    }
    const int64_t n_win = (int64_t)n_fields * ny * nx;
    int64_t blocks = (n_win + 7) / 8;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_window_gather4<<<(unsigned)blocks, 256, 0, s>>>(
        reinterpret_cast<const float4 *>(cells), valid, n_fields, ny, nx, dc / 4, gx, gy, t,
        last_ix, last_iy, reinterpret_cast<float4 *>(dense), ok);
    return cudaGetLastError();
  }
  dim3 grid((unsigned)(nx < 64 ? nx : 64), (unsigned)ny, (unsigned)n_fields);
  k_window_gather<<<grid, 128, 0, s>>>(cells, valid, ny, nx, dc, gx, gy, grid_step, last_ix,
                                       last_iy, dense, ok);
  return cudaGetLastError();
}

cudaError_t launch_mask_no_class(float *scores, const uint8_t *ok, int n_parts,
                                 int64_t n_per_part, cudaStream_t s) {
  k_mask_no_class<<<(unsigned)((n_per_part + 255) / 256), 256, 0, s>>>(scores, ok, n_per_part,
                                                                      n_parts);
  return cudaGetLastError();
}

}  // namespace pa
