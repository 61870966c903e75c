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
// KC: the most root children of the images; U: cells per thread and step.
template <int KC, int U>
__global__ void __launch_bounds__(kThreads) k_root_combine(const RootDesc *__restrict__ rds,
                                                           int64_t N) {
  root_combine_cells<KC, U>(rds[blockIdx.y], (int64_t)blockIdx.x * blockDim.x, N,
                            (int64_t)gridDim.x * blockDim.x);
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

// ---------------------------------------------------------------------------
// Log-partition log(sum_i exp(x_i)) of each map, accurate to double.
//
// GB300 runs FP64 at 1/64 of the FP32 rate, so one double operation per cell
// would cost more than the rest of the reduction; the sum is carried in
// float-float arithmetic instead (value = hi + lo, about 48 significant
// bits; Knuth's TwoSum, Dekker's Fast2Sum and the FMA TwoProduct as
// error-free transforms), and the per-block partials are combined in double.
//
// Each term t = exp(x - M) with M the map's maximum (from its argmax key):
//   y = x - M exactly as the float-float (s, e) (TwoSum),
//   n = round(64 s) (by the 1.5 * 2^23 rounding constant), r = (s - n/64) + e
//       with |r| <= 1/128 (s - n/64 is exact by Sterbenz's lemma), renormalised,
//   t = T[n] * (1 + p),  p = r + r^2/2 + r^3/6 + r^4/24 + r^5/120,
// where T[n] = exp(n/64) for n in [-kExpTabN, 0] comes from the table kernel
// (FP64 exp rounded to float-float).  The dropped Taylor terms are below
// 3e-16 of t and the float-rounded r^3.. terms contribute ~1e-14 of t.
// Cells with y <= -kExpTabN/64 take expf (their whole sum is below
// N * exp(-36), so its 1e-7 relative error is negligible).  Thread, warp and
// block orders are fixed, so the result is deterministic.
// ---------------------------------------------------------------------------
constexpr int kExpTabN = 36 * 64;  // T[n], n in [-kExpTabN, 0]

struct ff {
  float hi, lo;
};

// Knuth's TwoSum: a + b = s + e exactly.
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// |a| >= |b|: a + b = s + e exactly.
__device__ __forceinline__ ff quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
// tab[k] = exp(-k / 64) as float-float, k = 0..kExpTabN.
__global__ void k_exp_table(float2 *__restrict__ tab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k > kExpTabN) return;
  const double v = exp(-(double)k / 64.0);
  const float hi = __double2float_rn(v);
  tab[k] = make_float2(hi, __double2float_rn(v - (double)hi));
}

__global__ void __launch_bounds__(kThreads) k_log_z_partial(const float *const *__restrict__ maps,
                                                            const unsigned long long *__restrict__ amax,
                                                            int64_t N, const float2 *__restrict__ tab,
                                                            double *__restrict__ partials) {
  __shared__ float2 st[kExpTabN + 1];
  for (int k = threadIdx.x; k <= kExpTabN; k += blockDim.x) st[k] = tab[k];
  __syncthreads();
  const int map = blockIdx.y;
  const float *x = maps[map];
  const float M = ukey_decode((uint32_t)(amax[map] >> 32));
  constexpr float kMagic = 12582912.f;  // 1.5 * 2^23: x + kMagic rounds x to an integer
  ff acc{0.f, 0.f};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const ff y = two_sum(__ldg(x + i), -M);  // x - M exactly
    float th, tl;                            // the term as th + tl
    if (y.hi > -(float)(kExpTabN / 64)) {
      // n = round(64 y.hi) in [-kExpTabN, 0] (y <= 0: M is the maximum;
      // the clamp only guards the table index)
      const float t = __fmaf_rn(y.hi, 64.f, kMagic);
      const int n = min(0, max(-kExpTabN, __float_as_int(t) - __float_as_int(kMagic)));
      const float nf = __fsub_rn(t, kMagic);
      // r = (y.hi - n/64) + y.lo, the first difference exact (Sterbenz)
      const ff r = two_sum(__fmaf_rn(nf, -1.f / 64.f, y.hi), y.lo);
      // exp(r) - 1 = r + r^2/2 + c as ph + pl: r^2 = r2h + r2l exactly (FMA),
      // c = r^3/6 + r^4/24 + r^5/120 and the cross term r.hi * r.lo in float
      const float r2h = __fmul_rn(r.hi, r.hi);
      const float r2l = __fmaf_rn(r.hi, r.hi, -r2h);
      const float c = __fmul_rn(__fmul_rn(r.hi, r2h),
                                __fmaf_rn(r.hi, __fmaf_rn(r.hi, 1.f / 120.f, 1.f / 24.f), 1.f / 6.f));
      const float u = __fmaf_rn(r.hi, r.lo, __fmaf_rn(r2l, 0.5f, c));
      const ff v = two_sum(__fmul_rn(r2h, 0.5f), u);  // r^2/2 + c
      ff pp = quick_two_sum(r.hi, v.hi);               // |r| >= r^2/2 + c
      pp.lo = __fadd_rn(pp.lo, __fadd_rn(v.lo, r.lo));
      // term = T (1 + p) = T.hi + T.hi p + T.lo (1 + p); |T.hi p| <= T.hi / 128
      const float2 T = st[-n];
      const float q = __fmul_rn(T.x, pp.hi);
      const float qe = __fmaf_rn(T.x, pp.hi, -q);
      const float small = __fadd_rn(__fmaf_rn(T.x, pp.lo, __fmaf_rn(T.y, pp.hi, qe)), T.y);
      const ff tt = quick_two_sum(T.x, q);
      th = tt.hi;
      tl = __fadd_rn(tt.lo, small);
    } else {
      th = expf(y.hi);  // below exp(-36): the tail's 1e-7 relative error is negligible
      tl = 0.f;
    }
    // acc += (th, tl)
    ff s1 = two_sum(acc.hi, th);
    s1.lo = __fadd_rn(s1.lo, __fadd_rn(acc.lo, tl));
    acc = quick_two_sum(s1.hi, s1.lo);
  }
  double d = (double)acc.hi + (double)acc.lo;
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

cudaError_t launch_root_combine(const RootDesc *rd, int n_roots, int64_t N, int max_k,
                                cudaStream_t s) {
  int blocks = (int)((N + kThreads - 1) / kThreads);
  if (blocks > 152 * 4) blocks = 152 * 4;
  dim3 grid((unsigned)blocks, (unsigned)n_roots);
  if (max_k <= 8)  // four cells per thread and step, their loads in flight together
    k_root_combine<8, 4><<<grid, kThreads, 0, s>>>(rd, N);
  else
    k_root_combine<kMaxRootChildren, 1><<<grid, kThreads, 0, s>>>(rd, N);
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

size_t log_z_scratch_bytes(int n_maps) {
  return (size_t)n_maps * kLogZBlocks * sizeof(double) + (size_t)(kExpTabN + 1) * sizeof(float2);
}

cudaError_t launch_log_z(const float *const *maps, const unsigned long long *amax, int n_maps,
                         int64_t N, void *scratch, double *log_z, cudaStream_t s) {
  double *partials = static_cast<double *>(scratch);
  float2 *tab = reinterpret_cast<float2 *>(partials + (size_t)n_maps * kLogZBlocks);
  k_exp_table<<<(kExpTabN + 256) / 256, 256, 0, s>>>(tab);
  dim3 grid((unsigned)kLogZBlocks, (unsigned)n_maps);
  k_log_z_partial<<<grid, kThreads, 0, s>>>(maps, amax, N, tab, partials);
  k_log_z_final<<<(n_maps + 127) / 128, 128, 0, s>>>(partials, kLogZBlocks, amax, n_maps, log_z);
  return cudaGetLastError();
}

}  // namespace pa
