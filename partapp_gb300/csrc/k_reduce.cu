// k_reduce.cu -- root accumulation, root rotation marginalisation and the
// FP64 log-partition of each marginal.
#include "pa_internal.cuh"

namespace pa {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// Root of the tree.  In computeRootPosteriorRot (libPictStruct/
// objectdetect_findrot.cpp:630-654) every message from a root child is added
// into post[root] and into log_from_root of every *other* root child, in
// joint order, starting from zero-initialised grids; then the root unary is
// added to post[root], and computePartMarginals (:163-165) adds it to each
// log_from_root.  This kernel performs those sums element-wise in that order
// and folds the maxima that the downward messages need and the argmax of the
// root marginal (:261-277).
__global__ void __launch_bounds__(kThreads) k_root_combine(const RootDesc *__restrict__ rds,
                                                           int64_t N) {
  const RootDesc &rd = rds[blockIdx.y];
  const int k = rd.k;
  int keys[kMaxRootChildren];
#pragma unroll
  for (int c = 0; c < kMaxRootChildren; ++c) keys[c] = kFkeyNegInf;
  unsigned long long am = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    float m[kMaxRootChildren];
#pragma unroll
    for (int c = 0; c < kMaxRootChildren; ++c)
      if (c < k) m[c] = __ldg(rd.msg[c] + i);
    const float u = __ldg(rd.unary + i);
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kMaxRootChildren; ++c)
      if (c < k) s = __fadd_rn(s, m[c]);
    const float post = __fadd_rn(s, u);
    rd.post[i] = post;
    am = umax64(am, akey(post, (uint32_t)i));
#pragma unroll
    for (int j = 0; j < kMaxRootChildren; ++j) {
      if (j >= k) break;
      float fr = 0.f;
#pragma unroll
      for (int c = 0; c < kMaxRootChildren; ++c)
        if (c < k && c != j) fr = __fadd_rn(fr, m[c]);
      fr = __fadd_rn(fr, u);
      rd.from_root[j][i] = fr;
      keys[j] = max(keys[j], (fr == fr) ? fkey(fr) : kFkeyNegInf);
    }
  }
  __shared__ int skeys[kThreads / 32][kMaxRootChildren];
  __shared__ unsigned long long sam[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kMaxRootChildren; ++j) {
    const int v = __reduce_max_sync(0xFFFFFFFFu, keys[j]);
    if (lane == 0) skeys[warp][j] = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) am = umax64(am, __shfl_xor_sync(0xFFFFFFFFu, am, o));
  if (lane == 0) sam[warp] = am;
  __syncthreads();
  if (threadIdx.x < k) {
    int v = kFkeyNegInf;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = max(v, skeys[w][threadIdx.x]);
    atomicMax(rd.fr_max[threadIdx.x], v);
  }
  if (threadIdx.x == 0 && rd.amax) {
    unsigned long long b = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = umax64(b, sam[w]);
    atomicMax(rd.amax, b);
  }
}

// Root posterior over the kept rotations (objectdetect_findrot.cpp:694-726):
// exp of the first kept slice, += exp of each further kept slice, then
// computeLogGrid (0 -> LOG_ZERO).
__global__ void __launch_bounds__(kThreads) k_root_posterior(const float *const *__restrict__ post,
                                                             float *const *__restrict__ out,
                                                             const int *__restrict__ keep,
                                                             int n_keep, int HW) {
  const float *p = post[blockIdx.y];
  float *o = out[blockIdx.y];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < HW; i += gridDim.x * blockDim.x) {
    float e = expf(__ldg(p + (int64_t)keep[0] * HW + i));
    for (int k = 1; k < n_keep; ++k) e = __fadd_rn(e, expf(__ldg(p + (int64_t)keep[k] * HW + i)));
    o[i] = (e == 0.f) ? kLogZero : logf(e);
  }
}

// log(sum_i exp(x_i)) of each map, in double.  With M the map's maximum
// (from its argmax key) every term exp(x_i - M) lies in [0, 1]; each thread
// keeps a compensated (Kahan) float sum of its terms, blocks and maps are
// combined in double in a fixed order, so the result is deterministic.
__global__ void __launch_bounds__(kThreads) k_log_z_partial(const float *const *__restrict__ maps,
                                                            const unsigned long long *__restrict__ amax,
                                                            int64_t N, double *__restrict__ partials) {
  const int map = blockIdx.y;
  const float *x = maps[map];
  const float M = ukey_decode((uint32_t)(amax[map] >> 32));
  float s = 0.f, c = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float t = expf(__fsub_rn(__ldg(x + i), M));
    const float yk = __fsub_rn(t, c);
    const float tt = __fadd_rn(s, yk);
    c = __fsub_rn(__fsub_rn(tt, s), yk);
    s = tt;
  }
  double d = (double)s - (double)c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xFFFFFFFFu, d, o);
  __shared__ double sd[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sd[warp] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sd[w];
    partials[(int64_t)map * gridDim.x + blockIdx.x] = t;
  }
}

__global__ void k_log_z_final(const double *__restrict__ partials, int nb,
                              const unsigned long long *__restrict__ amax, int n_maps,
                              double *__restrict__ log_z) {
  const int map = blockIdx.x * blockDim.x + threadIdx.x;
  if (map >= n_maps) return;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += partials[(int64_t)map * nb + b];
  const double M = (double)ukey_decode((uint32_t)(amax[map] >> 32));
  log_z[map] = M + log(t);
}

// First-maximum argmax of whole maps (objectdetect_findrot.cpp:261-277).
__global__ void __launch_bounds__(kThreads) k_argmax(const float *const *__restrict__ maps,
                                                     int64_t N,
                                                     unsigned long long *__restrict__ amax) {
  const float *x = maps[blockIdx.y];
  unsigned long long am = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x)
    am = umax64(am, akey(__ldg(x + i), (uint32_t)i));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) am = umax64(am, __shfl_xor_sync(0xFFFFFFFFu, am, o));
  __shared__ unsigned long long sam[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sam[warp] = am;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = umax64(b, sam[w]);
    atomicMax(amax + blockIdx.y, b);
  }
}

}  // namespace

cudaError_t launch_argmax(const float *const *maps, int n_maps, int64_t N,
                          unsigned long long *amax, cudaStream_t s) {
  dim3 grid(152u, (unsigned)n_maps);
  k_argmax<<<grid, kThreads, 0, s>>>(maps, N, amax);
  return cudaGetLastError();
}

cudaError_t launch_root_combine(const RootDesc *rd, int n_roots, int64_t N, cudaStream_t s) {
  int blocks = (int)((N + kThreads - 1) / kThreads);
  if (blocks > 152 * 4) blocks = 152 * 4;
  dim3 grid((unsigned)blocks, (unsigned)n_roots);
  k_root_combine<<<grid, kThreads, 0, s>>>(rd, N);
  return cudaGetLastError();
}

cudaError_t launch_root_posterior(const float *const *post_root, float *const *root_post,
                                  const int *keep, int n_keep, int n_images, int R, int H, int W,
                                  cudaStream_t s) {
  (void)R;
  const int HW = H * W;
  int blocks = (HW + kThreads - 1) / kThreads;
  if (blocks > 304) blocks = 304;
  dim3 grid((unsigned)blocks, (unsigned)n_images);
  k_root_posterior<<<grid, kThreads, 0, s>>>(post_root, root_post, keep, n_keep, HW);
  return cudaGetLastError();
}

cudaError_t launch_log_z(const float *const *maps, const unsigned long long *amax, int n_maps,
                         int64_t N, double *partials, double *log_z, cudaStream_t s) {
  dim3 grid((unsigned)kLogZBlocks, (unsigned)n_maps);
  k_log_z_partial<<<grid, kThreads, 0, s>>>(maps, amax, N, partials);
  k_log_z_final<<<(n_maps + 127) / 128, 128, 0, s>>>(partials, kLogZBlocks, amax, n_maps, log_z);
  return cudaGetLastError();
}

}  // namespace pa
