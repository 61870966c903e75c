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
