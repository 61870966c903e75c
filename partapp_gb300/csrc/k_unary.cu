// k_unary.cu -- score grids -> masked log unary maps.
//
// Per (part, rotation) map this fuses, in the reference's order:
//   transform_grid_fixed_size(grid -> image, Tig, NO_CLASS_VALUE, method)
//       (libMultiArray/multi_array_transform.hpp:123-257, called from
//        PartApp::loadScoreGrid, libPartApp/partapp.cpp:887-896, and
//        partdetect_dense, libPartDetect/partdetect_test.cpp:283-289)
//   clip_scores_fill          (libPictStruct/objectdetect_aux.hpp:42-60)
//   computeLogGrid            (libMultiArray/multi_array_op.hpp:154-167)
//   upright mask, root strip  (libPictStruct/objectdetect_findrot.cpp:509-551)
// and folds the map's maximum (getMinMax of the first message,
// multi_array_op.hpp:61-77) into one atomic per CTA.
//
// Grid coordinates are evaluated in double with the reference's rounding
// (explicit __dmul_rn/__dadd_rn: no fused multiply-add); for axis-aligned Tig
// the per-column / per-row coordinates come from host-built tables.
#include "pa_internal.cuh"

namespace pa {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float clip_log(float v) {
  if (v < 0.f) v = kClipMin;
  return v == 0.f ? kLogZero : logf(v);
}

__device__ __forceinline__ void block_max_commit(int key, int *slot) {
  key = __reduce_max_sync(0xFFFFFFFFu, key);
  __shared__ int wmax[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) wmax[warp] = key;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = wmax[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = max(m, wmax[w]);
    atomicMax(slot, m);
  }
}

__device__ __forceinline__ int key_of(float v) { return (v == v) ? fkey(v) : kFkeyNegInf; }

// TM_BILINEAR: one CTA per (map, band of rows).
__global__ void __launch_bounds__(kThreads) k_unary_bilinear(const UnaryMap *__restrict__ maps,
                                                             int ny, int nx, int H, int W,
                                                             int rows_per_cta) {
  const UnaryMap m = maps[blockIdx.x];
  const int y0 = blockIdx.y * rows_per_cta;
  const int y1e = min(H, y0 + rows_per_cta);
  const float eps10 = 10.0f * 1.1920928955078125e-07f;  // 10 * FLT_EPSILON
  int kmax = kFkeyNegInf;
  const int npix = (y1e - y0) * W;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) {
    const int y3 = y0 + i / W, x3 = i - (i / W) * W;
    float v = kNoClassValue;
    int ix1, iy1;
    float a, b;
    if (m.separable) {
      ix1 = m.colx[x3];
      a = m.cola[x3];
      iy1 = m.rowy[y3];
      b = m.rowb[y3];
    } else {
      const double x1 = __dadd_rn(__dadd_rn(__dmul_rn(m.T13[0], (double)x3), __dmul_rn(m.T13[1], (double)y3)), m.T13[2]);
      const double yy = __dadd_rn(__dadd_rn(__dmul_rn(m.T13[3], (double)x3), __dmul_rn(m.T13[4], (double)y3)), m.T13[5]);
      ix1 = (int)floor(x1);
      iy1 = (int)floor(yy);
      a = __double2float_rn(__dsub_rn(x1, (double)ix1));
      b = __double2float_rn(__dsub_rn(yy, (double)iy1));
    }
    if (ix1 >= 0 && ix1 < nx && iy1 >= 0 && iy1 < ny) {
      const float *g0 = m.grid + (int64_t)iy1 * nx + ix1;
      if (a < eps10 && b < eps10) {
        v = __ldg(g0);
      } else if (ix1 < nx - 1 && iy1 < ny - 1) {
        const float *g1 = g0 + nx;
        const float omb = __fsub_rn(1.0f, b), oma = __fsub_rn(1.0f, a);
        const float t0 = __fmul_rn(__fmul_rn(omb, oma), __ldg(g0));
        const float t1 = __fmul_rn(__fmul_rn(omb, a), __ldg(g0 + 1));
        const float t2 = __fmul_rn(__fmul_rn(b, oma), __ldg(g1));
        const float t3 = __fmul_rn(__fmul_rn(b, a), __ldg(g1 + 1));
        v = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
      }
    }
    float o = clip_log(v);
    if (m.masked_all || (m.strip > 0 && (x3 < m.strip || x3 >= W - m.strip))) o = kLogZero;
    m.out[(int64_t)y3 * W + x3] = o;
    kmax = max(kmax, key_of(o));
  }
  if (m.max_slot) block_max_commit(kmax, m.max_slot);
}

// TM_BILINEAR with axis-aligned Tig: per (map, band of rows) the column
// table and the few grid rows the band reads are staged in shared memory.
__global__ void __launch_bounds__(kThreads) k_unary_bilinear_sep(const UnaryMap *__restrict__ maps,
                                                                 int ny, int nx, int H, int W,
                                                                 int rows_per_cta) {
  extern __shared__ __align__(16) float sm[];
  const UnaryMap &mg = maps[blockIdx.x];
  const float *grid = mg.grid;
  float *out = mg.out;
  const int *colx = mg.colx, *rowy = mg.rowy;
  const float *cola = mg.cola, *rowb = mg.rowb;
  const int masked_all = mg.masked_all, strip = mg.strip;
  int *max_slot = mg.max_slot;
  const int y0 = blockIdx.y * rows_per_cta;
  const int y1e = min(H, y0 + rows_per_cta);
  const float eps10 = 10.0f * 1.1920928955078125e-07f;  // 10 * FLT_EPSILON
  if (masked_all) {  // every output is LOG_ZERO (uniform for the CTA)
    for (int i = threadIdx.x; i < (y1e - y0) * W; i += blockDim.x) out[(int64_t)y0 * W + i] = kLogZero;
    if (max_slot) block_max_commit(fkey(kLogZero), max_slot);
    return;
  }
  int *sx = reinterpret_cast<int *>(sm);          // [W] ix1
  float *sa = sm + W;                             // [W] a
  float *sg = sm + 2 * W;                         // [nrows][nx] grid rows
  // grid rows read by this band: [rlo, rhi] (rows are monotone in y3)
  int rlo = rowy[y0], rhi = rowy[y1e - 1];
  if (rlo > rhi) { const int t = rlo; rlo = rhi; rhi = t; }
  rlo = max(rlo, 0);
  rhi = min(rhi + 1, ny - 1);
  const int nrows = rhi >= rlo ? rhi - rlo + 1 : 0;
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    sx[i] = colx[i];
    sa[i] = cola[i];
  }
  for (int i = threadIdx.x; i < nrows * nx; i += blockDim.x) sg[i] = __ldg(grid + (int64_t)rlo * nx + i);
  __syncthreads();
  // running maximum as a float: fmaxf skips NaN (key_of's -inf) and the
  // outputs are never -0 (logf gives +0 at 1), so key_of(omax) is the
  // maximum of the outputs' keys
  float omax = -INFINITY;
  for (int y3 = y0; y3 < y1e; ++y3) {
    const int iy1 = rowy[y3];
    const float b = rowb[y3];
    const bool yin = (iy1 >= 0 && iy1 < ny);
    for (int x3 = threadIdx.x; x3 < W; x3 += blockDim.x) {
      float v = kNoClassValue;
      const int ix1 = sx[x3];
      const float a = sa[x3];
      if (yin && ix1 >= 0 && ix1 < nx) {
        const float *g0 = sg + (iy1 - rlo) * nx + ix1;
        if (a < eps10 && b < eps10) {
          v = g0[0];
        } else if (ix1 < nx - 1 && iy1 < ny - 1) {
          const float *g1 = g0 + nx;
          const float omb = __fsub_rn(1.0f, b), oma = __fsub_rn(1.0f, a);
          const float t0 = __fmul_rn(__fmul_rn(omb, oma), g0[0]);
          const float t1 = __fmul_rn(__fmul_rn(omb, a), g0[1]);
          const float t2 = __fmul_rn(__fmul_rn(b, oma), g1[0]);
          const float t3 = __fmul_rn(__fmul_rn(b, a), g1[1]);
          v = __fadd_rn(__fadd_rn(__fadd_rn(t0, t1), t2), t3);
        }
      }
      float o = clip_log(v);
      if (strip > 0 && (x3 < strip || x3 >= W - strip)) o = kLogZero;
      out[(int64_t)y3 * W + x3] = o;
      omax = fmaxf(omax, o);
    }
  }
  if (max_slot) block_max_commit(key_of(omax), max_slot);
}

// TM_DIRECT, pass 1: every pixel starts at NO_CLASS_VALUE -> LOG_ZERO.
__global__ void __launch_bounds__(kThreads) k_unary_direct_fill(const UnaryMap *__restrict__ maps,
                                                                int H, int W, int rows_per_cta) {
  const UnaryMap m = maps[blockIdx.x];
  const int y0 = blockIdx.y * rows_per_cta;
  const int y1e = min(H, y0 + rows_per_cta);
  const int npix = (y1e - y0) * W;
  if (m.order) {  // ordered map: the gather pass writes every pixel
    int *ord = m.order + (int64_t)y0 * W;
    for (int i = threadIdx.x; i < npix; i += blockDim.x) ord[i] = -1;
    return;
  }
  float *out = m.out + (int64_t)y0 * W;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) out[i] = kLogZero;
  if (m.max_slot && blockIdx.y == 0) block_max_commit(fkey(kLogZero), m.max_slot);
}

// TM_DIRECT, pass 2: forward-map every grid cell != NO_CLASS_VALUE
// (multi_array_transform.hpp:173-193).  An injective map writes the pixel
// directly.  Where two cells may land on one pixel the reference keeps the
// last one its loop (x1 outer, y1 inner) writes: the cell's position in that
// loop, x1 * ny + y1, goes to the pixel by atomicMax and pass 3 reads the
// winner.  A squeezed grid's loop runs over a sub-box of the same cells in
// the same (x1, y1) order, so the full grid's index orders it too.
__global__ void __launch_bounds__(kThreads) k_unary_direct_scatter(const UnaryMap *__restrict__ maps,
                                                                   int ny, int nx, int H, int W) {
  const UnaryMap m = maps[blockIdx.x];
  int kmax = kFkeyNegInf;
  for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < ny * nx; i += gridDim.y * blockDim.x) {
    const int y1 = i / nx, x1 = i - y1 * nx;
    const float v = __ldg(m.grid + i);
    if (v == kNoClassValue) continue;
    int ix3, iy3;
    if (m.separable) {
      ix3 = m.colx[x1];
      iy3 = m.rowy[y1];
    } else {
      const double xs = (double)(x1 - m.ox), ys = (double)(y1 - m.oy);
      const double x3 = __dadd_rn(__dadd_rn(__dmul_rn(m.T31[0], xs), __dmul_rn(m.T31[1], ys)), m.T31[2]);
      const double y3 = __dadd_rn(__dadd_rn(__dmul_rn(m.T31[3], xs), __dmul_rn(m.T31[4], ys)), m.T31[5]);
      ix3 = (int)floor(__dadd_rn(x3, 0.5));
      iy3 = (int)floor(__dadd_rn(y3, 0.5));
    }
    if (ix3 < 0 || ix3 >= W || iy3 < 0 || iy3 >= H) continue;
    if (m.order) {
      atomicMax(m.order + (int64_t)iy3 * W + ix3, x1 * ny + y1);
      continue;
    }
    float o = clip_log(v);
    if (m.masked_all || (m.strip > 0 && (ix3 < m.strip || ix3 >= W - m.strip))) o = kLogZero;
    m.out[(int64_t)iy3 * W + ix3] = o;
    kmax = max(kmax, key_of(o));
  }
  if (m.max_slot && !m.order) block_max_commit(kmax, m.max_slot);
}

// TM_DIRECT, pass 3 of an ordered map: each pixel takes its last writer's
// value (NO_CLASS_VALUE -> LOG_ZERO where no cell landed).
__global__ void __launch_bounds__(kThreads) k_unary_direct_gather(const UnaryMap *__restrict__ maps,
                                                                  int ny, int nx, int H, int W,
                                                                  int rows_per_cta) {
  const UnaryMap m = maps[blockIdx.x];
  if (!m.order) return;
  const int y0 = blockIdx.y * rows_per_cta;
  const int y1e = min(H, y0 + rows_per_cta);
  const int npix = (y1e - y0) * W;
  const int *ord = m.order + (int64_t)y0 * W;
  float *out = m.out + (int64_t)y0 * W;
  int kmax = kFkeyNegInf;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) {
    const int k = ord[i];
    float o = kLogZero;
    if (k >= 0) {
      const int x1 = k / ny, y1 = k - x1 * ny;
      const int x3 = i % W;
      o = clip_log(__ldg(m.grid + (int64_t)y1 * nx + x1));
      if (m.masked_all || (m.strip > 0 && (x3 < m.strip || x3 >= W - m.strip))) o = kLogZero;
    }
    out[i] = o;
    kmax = max(kmax, key_of(o));
  }
  if (m.max_slot) block_max_commit(kmax, m.max_slot);
}

// Upright mask + root strip applied to caller-provided log unaries, with the
// part maximum.  masked_rot[r] != 0 marks a rotation the upright rule drops.
__global__ void __launch_bounds__(kThreads) k_prepare_unary(const float *__restrict__ in,
                                                            float *__restrict__ out,
                                                            const int *__restrict__ masked_rot,
                                                            int strip, int R, int H, int W,
                                                            int *max_slot) {
  const int64_t HW = (int64_t)H * W;
  const int64_t N = HW * R;
  int kmax = kFkeyNegInf;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / HW);
    const int x = (int)(i % W);
    float o = in[i];
    if ((masked_rot && masked_rot[r]) || (strip > 0 && (x < strip || x >= W - strip))) o = kLogZero;
    out[i] = o;
    kmax = max(kmax, key_of(o));
  }
  if (max_slot) block_max_commit(kmax, max_slot);
}

__global__ void __launch_bounds__(kThreads) k_map_max(const float *__restrict__ x, int64_t N,
                                                      int *max_slot) {
  int kmax = kFkeyNegInf;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x)
    kmax = max(kmax, key_of(__ldg(x + i)));
  block_max_commit(kmax, max_slot);
}

// Copies n 16-byte words; the source may be pinned host memory (unified
// addressing), which keeps small uploads off the copy engines.
__global__ void k_copy16(const int4 *__restrict__ src, int4 *__restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

__global__ void k_fill_int(int *p, int v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

}  // namespace

cudaError_t launch_unary_maps(const UnaryMap *maps, int n_maps, int ny, int nx, int H, int W,
                              int direct, int separable, int ordered, cudaStream_t s) {
  const int rows = 16;
  dim3 grid((unsigned)n_maps, (unsigned)((H + rows - 1) / rows));
  if (!direct) {
    // rows of the grid one band reads: at most rows * |dy1/dy3| + 2
    const size_t smem = (size_t)(2 * W + (size_t)(rows + 2) * nx) * sizeof(float);
    if (separable && smem <= 96 * 1024) {
      cudaFuncSetAttribute(k_unary_bilinear_sep, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
      k_unary_bilinear_sep<<<grid, kThreads, smem, s>>>(maps, ny, nx, H, W, rows);
    } else {
      k_unary_bilinear<<<grid, kThreads, 0, s>>>(maps, ny, nx, H, W, rows);
    }
  } else {
    k_unary_direct_fill<<<grid, kThreads, 0, s>>>(maps, H, W, rows);
    // cells of a map spread over several CTAs (injective map: no write order)
    int chunks = (ny * nx + 8 * kThreads - 1) / (8 * kThreads);
    if (chunks > 64) chunks = 64;
    k_unary_direct_scatter<<<dim3((unsigned)n_maps, (unsigned)chunks), kThreads, 0, s>>>(
        maps, ny, nx, H, W);
    if (ordered) k_unary_direct_gather<<<grid, kThreads, 0, s>>>(maps, ny, nx, H, W, rows);
  }
  return cudaGetLastError();
}

cudaError_t launch_prepare_unary(const float *in, float *out, const int *masked_rot, int strip,
                                 int R, int H, int W, int *max_slot, cudaStream_t s) {
  const int64_t N = (int64_t)R * H * W;
  int blocks = (int)((N + kThreads - 1) / kThreads);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_prepare_unary<<<blocks, kThreads, 0, s>>>(in, out, masked_rot, strip, R, H, W, max_slot);
  return cudaGetLastError();
}

cudaError_t launch_map_max(const float *x, int64_t N, int *max_slot, cudaStream_t s) {
  int blocks = (int)((N + kThreads - 1) / kThreads);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_map_max<<<blocks, kThreads, 0, s>>>(x, N, max_slot);
  return cudaGetLastError();
}

cudaError_t launch_copy16(const void *src, void *dst, int64_t n_words, cudaStream_t s) {
  int blocks = (int)((n_words + 255) / 256);
  if (blocks > 256) blocks = 256;
  if (blocks < 1) blocks = 1;
  k_copy16<<<blocks, 256, 0, s>>>(reinterpret_cast<const int4 *>(src), reinterpret_cast<int4 *>(dst),
                                  n_words);
  return cudaGetLastError();
}

cudaError_t launch_fill_int(int *p, int v, int64_t n, cudaStream_t s) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  k_fill_int<<<blocks, 256, 0, s>>>(p, v, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Poselet-conditioned extra unaries of findObjectImageRotJoints
// (libPictStruct/objectdetect_findrot.cpp:915-948, the functions of
// objectdetect_icps.cpp), added to the log detections in the reference's
// order and typing:
//   rotation:  u = u + w_rot * rot_tab[p][r]           (getRotScoreGrid :228-281
//              + addExtraUnary :524-547, float products and sums)
//   position:  u = u + w_pos * log(max(gx * gy, 1e-4))  for parts != root
//              (getPosScoreGrid :366-448), gx = exp(-0.5 (x - det_x - mu_x)^2
//              / var_x) in double, rounded to float
//   torso:     u = u + log(max(w * gx * gy, 1e-4))     for the root part, the sum in
//              double (setTorsoPosPrior :137-191, relative to the image centre)
// One thread per (part, pixel), walking the part's scales and rotations.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gauss_term(float rel, float mu, float var) {
  const double d = (double)__fsub_rn(rel, mu);
  return (float)exp(-0.5 * (d * d) / (double)var);
}

__global__ void k_extra_unary(ExtraUnary ex, float *__restrict__ lu, int S, int R, int H, int W) {
  const int p = blockIdx.y;
  const int64_t HW = (int64_t)H * W;
  const int64_t pix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (pix >= HW) return;
  const int iy = (int)(pix / W), ix = (int)(pix - (int64_t)iy * W);
  const bool detect = ex.is_detect ? ex.is_detect[p] != 0 : true;
  const bool rot = ex.rot_on;
  // parts without a position score still get weight * 0 added (the zero
  // grids of addExtraUnary)
  float pos_w = __fmul_rn(ex.pos_weight, 0.f);
  const bool pos = ex.pos_on;
  if (ex.pos_on && detect && p != ex.root) {
    const float ixr = (float)((double)ix - ex.root_det_x), iyr = (float)((double)iy - ex.root_det_y);
    float sc = __fmul_rn(gauss_term(ixr, ex.pos[p].x, ex.pos[p].z), gauss_term(iyr, ex.pos[p].y, ex.pos[p].w));
    if ((double)sc < 1e-4) sc = 1e-4f;
    pos_w = __fmul_rn(ex.pos_weight, logf(sc));
  }
  bool torso = false;
  double torso_v = 0.0;
  if (ex.torso_on && p == ex.root) {
    const float ixr = __fsub_rn(ex.img_cx, (float)ix), iyr = __fsub_rn(ex.img_cy, (float)iy);
    float sc = __fmul_rn(__fmul_rn(ex.torso_weight, gauss_term(ixr, ex.torso.x, ex.torso.z)),
                         gauss_term(iyr, ex.torso.y, ex.torso.w));
    if ((double)sc < 1e-4) sc = 1e-4f;
    torso_v = (double)logf(sc);
    torso = true;
  }
  for (int s = 0; s < S; ++s)
    for (int r = 0; r < R; ++r) {
      float *c = lu + (((int64_t)p * S + s) * R + r) * HW + pix;
      float u = *c;
      if (rot) u = __fadd_rn(u, __fmul_rn(ex.rot_weight, ex.rot_tab[p * R + r]));
      if (pos) u = __fadd_rn(u, pos_w);
      if (torso) u = (float)((double)u + torso_v);
      *c = u;
    }
}

cudaError_t launch_extra_unary(const ExtraUnary &ex, float *lu, int P, int S, int R, int H, int W,
                               cudaStream_t s) {
  const int64_t HW = (int64_t)H * W;
  if (P < 1 || P > 65535 || HW < 1 || (HW + kThreads - 1) / kThreads > 0x7FFFFFFF)
    return cudaErrorInvalidValue;
  k_extra_unary<<<dim3((unsigned)((HW + kThreads - 1) / kThreads), (unsigned)P), kThreads, 0, s>>>(
      ex, lu, S, R, H, W);
  return cudaGetLastError();
}

// addLoadDPMScore's term (objectdetect_icps.cpp:476-482): val > 1e-4 compares
// in double, dpm_weight * log(val) is float (std::log(float)), log(1e-4) is
// double, so the conditional is double and the += rounds once to float.
__device__ __forceinline__ float add_loaded_dpm(float u, float val, float w, double log_floor) {
  const double t = (double)val > 1e-4 ? (double)__fmul_rn(w, logf(val)) : log_floor;
  return (float)((double)u + t);
}

// The DPM terms of findObjectImageRotJoints (objectdetect_findrot.cpp:883-914)
// in the reference's order: the torso grid, computeLogGrid'ed in float and
// added to the root part by addDPMScore (objectdetect_icps.cpp:488-522, float
// products and sums); the head grid (addLoadDPMScore for one part); the
// per-part unary grids (addLoadDPMScore for every detected part).  Thread per
// (part, pixel); every scale and rotation of that pixel in turn.
__global__ void k_dpm_score(DpmTerms dt, float *__restrict__ lu, int S, int R, int H, int W) {
  const int p = blockIdx.y;
  const int64_t HW = (int64_t)H * W;
  const int64_t pix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (pix >= HW) return;
  const bool detect = dt.is_detect ? dt.is_detect[p] != 0 : true;
  const bool torso = dt.torso && p == dt.root;
  float torso_w = 0.f;
  if (torso) {
    const float g = dt.torso[pix];
    if (!(g >= 0.f)) {  // computeLogGrid's domain: the call fails, the maps are undefined
      atomicOr(dt.err, 1);
      return;
    }
    torso_w = __fmul_rn(dt.torso_weight, g == 0.f ? (float)-1e6 : logf(g));
  }
  const bool head = dt.head && detect && p == dt.head_part;
  const float head_v = head ? dt.head[pix] : 0.f;
  const bool unary = dt.unary && detect;
  const int Ru = dt.unary_rot ? R : 1;
  for (int s = 0; s < S; ++s)
    for (int r = 0; r < R; ++r) {
      float *c = lu + (((int64_t)p * S + s) * R + r) * HW + pix;
      float u = *c;
      if (torso) u = __fadd_rn(u, torso_w);
      if (head) u = add_loaded_dpm(u, head_v, dt.head_weight, dt.log_floor);
      if (unary)
        u = add_loaded_dpm(u, dt.unary[((int64_t)p * Ru + (dt.unary_rot ? r : 0)) * HW + pix],
                           dt.unary_weight, dt.log_floor);
      *c = u;
    }
}

cudaError_t launch_dpm_score(const DpmTerms &dt, float *lu, int P, int S, int R, int H, int W,
                             cudaStream_t s) {
  const int64_t HW = (int64_t)H * W;
  if (P < 1 || P > 65535 || HW < 1 || (HW + kThreads - 1) / kThreads > 0x7FFFFFFF)
    return cudaErrorInvalidValue;
  k_dpm_score<<<dim3((unsigned)((HW + kThreads - 1) / kThreads), (unsigned)P), kThreads, 0, s>>>(
      dt, lu, S, R, H, W);
  return cudaGetLastError();
}

// nms_recursive (libPictStruct/objectdetect_aux.cpp:407-451): hypothesis j is
// suppressed when some earlier (higher-scored) hypothesis i lies inside i's
// ellipse, dx^2 / e1_i + dy^2 / e2_i < 1 with e1_i = (ellipse * scale_i *
// width)^2; whether i is itself suppressed does not matter, so every j is
// independent.  dx is the float difference of the float coordinates, widened;
// the rest is double, each operation rounded on its own (no fused multiply-add).
// A thread per j, the earlier hypotheses staged through shared memory in
// tiles.  err bit 1: scores not in descending order (the reference asserts).
constexpr int kNmsTile = 256;
__global__ void __launch_bounds__(kNmsTile) k_nms(const float *__restrict__ x, const float *__restrict__ y,
                                                 const float *__restrict__ scale, const float *__restrict__ score,
                                                 int n, double ew, double eh, int *__restrict__ out,
                                                 int *__restrict__ err) {
  __shared__ float sx[kNmsTile], sy[kNmsTile];
  __shared__ double se1[kNmsTile], se2[kNmsTile];
  const int j = blockIdx.x * kNmsTile + threadIdx.x;
  const bool live = j < n;
  const float xj = live ? x[j] : 0.f, yj = live ? y[j] : 0.f;
  if (live && j + 1 < n && score[j] < score[j + 1]) atomicOr(err, 1);
  bool sup = false;
  const int i_end = min(n, (int)(blockIdx.x + 1) * kNmsTile);  // the block's last j + 1
  for (int t0 = 0; t0 < i_end; t0 += kNmsTile) {
    __syncthreads();
    const int i = t0 + threadIdx.x;
    if (i < n) {
      sx[threadIdx.x] = x[i];
      sy[threadIdx.x] = y[i];
      const double sc = (double)scale[i];
      const double a = __dmul_rn(__dmul_rn(0.5, sc), ew), b = __dmul_rn(__dmul_rn(0.5, sc), eh);
      se1[threadIdx.x] = __dmul_rn(a, a);
      se2[threadIdx.x] = __dmul_rn(b, b);
    }
    __syncthreads();
    const int m = min(kNmsTile, j - t0);  // earlier hypotheses of this tile
    for (int k = 0; k < m && !sup; ++k) {
      const double dx = (double)__fsub_rn(sx[k], xj), dy = (double)__fsub_rn(sy[k], yj);
      const double q = __dadd_rn(__ddiv_rn(__dmul_rn(dx, dx), se1[k]), __ddiv_rn(__dmul_rn(dy, dy), se2[k]));
      sup = q < 1.0;
    }
  }
  if (live) out[j] = sup ? 1 : 0;
}

// nms_recursive of libNms, rectangle form (libNms/nms.cpp:132-225): rectangle
// i suppresses every later rectangle j whose centre, projected on i's unit
// edges v1 = r1 - r0 and v2 = r1 - r2, has dx^2 / e1 + dy^2 / e2 < thr with
// e1 = |r1 - r0|^2, e2 = |r1 - r2|^2 (all in double, each operation rounded
// as the reference's QPointF arithmetic rounds it).  One thread per j;
// earlier rectangles staged in 256-wide shared tiles.
__device__ __forceinline__ void rect_center(const double *r, double &cx, double &cy) {
  cx = __dmul_rn(0.25, __dadd_rn(__dadd_rn(__dadd_rn(r[0], r[2]), r[4]), r[6]));
  cy = __dmul_rn(0.25, __dadd_rn(__dadd_rn(__dadd_rn(r[1], r[3]), r[5]), r[7]));
}

__global__ void __launch_bounds__(kNmsTile) k_nms_rects(const double *__restrict__ rects,
                                                       const double *__restrict__ score, int n,
                                                       double thr, int *__restrict__ out,
                                                       int *__restrict__ err) {
  __shared__ double sc[2][kNmsTile], sv[4][kNmsTile], se[2][kNmsTile];
  const int j = blockIdx.x * kNmsTile + threadIdx.x;
  const bool live = j < n;
  double cxj = 0.0, cyj = 0.0;
  if (live) rect_center(rects + (int64_t)8 * j, cxj, cyj);
  if (live && j + 1 < n && score[j] < score[j + 1]) atomicOr(err, 1);
  bool sup = false;
  const int i_end = min(n, (int)(blockIdx.x + 1) * kNmsTile);  // the block's last j + 1
  for (int t0 = 0; t0 < i_end; t0 += kNmsTile) {
    __syncthreads();
    const int i = t0 + threadIdx.x;
    if (i < n) {
      const double *r = rects + (int64_t)8 * i;
      const double v1x = __dsub_rn(r[2], r[0]), v1y = __dsub_rn(r[3], r[1]);
      const double v2x = __dsub_rn(r[2], r[4]), v2y = __dsub_rn(r[3], r[5]);
      const double e1 = __dadd_rn(__dmul_rn(v1x, v1x), __dmul_rn(v1y, v1y));
      const double e2 = __dadd_rn(__dmul_rn(v2x, v2x), __dmul_rn(v2y, v2y));
      const double n1 = __dsqrt_rn(e1), n2 = __dsqrt_rn(e2);
      sv[0][threadIdx.x] = __ddiv_rn(v1x, n1);
      sv[1][threadIdx.x] = __ddiv_rn(v1y, n1);
      sv[2][threadIdx.x] = __ddiv_rn(v2x, n2);
      sv[3][threadIdx.x] = __ddiv_rn(v2y, n2);
      se[0][threadIdx.x] = e1;
      se[1][threadIdx.x] = e2;
      rect_center(r, sc[0][threadIdx.x], sc[1][threadIdx.x]);
    }
    __syncthreads();
    const int m = min(kNmsTile, j - t0);  // earlier rectangles of this tile
    for (int k = 0; k < m && !sup; ++k) {
      const double px = __dsub_rn(cxj, sc[0][k]), py = __dsub_rn(cyj, sc[1][k]);
      const double dx = __dadd_rn(__dmul_rn(sv[0][k], px), __dmul_rn(sv[1][k], py));
      const double dy = __dadd_rn(__dmul_rn(sv[2][k], px), __dmul_rn(sv[3][k], py));
      const double q =
          __dadd_rn(__ddiv_rn(__dmul_rn(dx, dx), se[0][k]), __ddiv_rn(__dmul_rn(dy, dy), se[1][k]));
      sup = q < thr;
    }
  }
  if (live) out[j] = sup ? 1 : 0;
}

cudaError_t launch_nms_rects(const double *rects, const double *score, int n, double thr, int *out,
                             int *err, cudaStream_t s) {
  if (n < 1) return cudaSuccess;
  k_nms_rects<<<(n + kNmsTile - 1) / kNmsTile, kNmsTile, 0, s>>>(rects, score, n, thr, out, err);
  return cudaGetLastError();
}

cudaError_t launch_nms(const float *x, const float *y, const float *scale, const float *score, int n,
                       double train_w, double train_h, int *out, int *err, cudaStream_t s) {
  if (n < 1) return cudaSuccess;
  k_nms<<<(n + kNmsTile - 1) / kNmsTile, kNmsTile, 0, s>>>(x, y, scale, score, n, train_w, train_h,
                                                          out, err);
  return cudaGetLastError();
}

}  // namespace pa
