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
                                                     int64_t n_loc, int dim, int dp,
                                                     int normalize, float *__restrict__ scores,
                                                     int n_fields) {
  extern __shared__ float sm[];
  const int field = blockIdx.y;
  const int64_t loc0 = (int64_t)blockIdx.x * kLoc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const float *src = desc + ((int64_t)field * n_loc + loc0) * dim;
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
    s += (__fmul_rn(val, q.y) < __fmul_rn(q.z, q.y)) ? q.w : -q.w;
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

__global__ void k_mask_no_class(float *__restrict__ scores, const uint8_t *__restrict__ ok,
                                int64_t n_per_part, int n_parts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_per_part) return;
  if (!ok[i])
    for (int p = 0; p < n_parts; ++p) scores[(int64_t)p * n_per_part + i] = kNoClassValue;
}

}  // namespace

cudaError_t launch_score_grids(const StumpPart *parts_dev, int n_parts, const float *desc,
                               int64_t n_loc, int n_fields, int dim, int normalize,
                               float *scores, cudaStream_t s) {
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
  k_score_grids<<<grid, 32 * gw, smem, s>>>(parts_dev, n_parts, desc, n_loc, dim, dp, normalize,
                                            scores, n_fields);
  return cudaGetLastError();
}

cudaError_t launch_window_gather(const float *cells, const uint8_t *valid, int n_fields, int ny,
                                 int nx, int dc, int gx, int gy, double grid_step, float *dense,
                                 uint8_t *ok, cudaStream_t s) {
  const int last_ix = nx - (int)floor(grid_step * (gx - 1) + 0.5) - 1;
  const int last_iy = ny - (int)floor(grid_step * (gy - 1) + 0.5) - 1;
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
