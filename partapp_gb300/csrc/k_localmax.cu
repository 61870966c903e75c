// k_localmax.cu -- findLocalMax (libPictStruct/objectdetect_aux.cpp:193-264).
//
// A cell (s, y, x) of a [S][H][W] grid is a local maximum when no in-grid
// 8-neighbour in its slice is strictly greater and, for S > 1, the cells of
// the adjacent slices s-1 and s+1 (no wrap-around) are strictly smaller.
// The reference enumerates maxima with s outermost, then x, then y; if more
// than max_n are found it keeps the max_n largest values (std::sort by value,
// descending; ties keep enumeration order here).
//
// GPU form: every local maximum becomes a 64-bit key whose high word orders
// the value and whose low word is ~enumeration index, so "larger key" is
// "larger value, then earlier in enumeration".  Chunks of kChunk keys are
// sorted in shared memory and cut to their top max_n; repeated levels shrink
// the candidate list until one chunk remains, which is ordered by key (more
// than max_n maxima) or by enumeration index (at most max_n maxima).
#include "pa_internal.cuh"

namespace pa {
namespace {

constexpr int kChunk = 4096;
constexpr int kThreads = 1024;

// Candidates of one (slice, 8-row x 32-column tile): the tile and a one-cell
// halo of the slice are staged in shared memory, the adjacent slices are
// read only at the cells that survive the in-slice test.
constexpr int kTY = 8, kTX = 32;

__global__ void __launch_bounds__(256) k_lm_cand(const float *const *__restrict__ maps, int S,
                                                 int H, int W,
                                                 unsigned long long *__restrict__ keys,
                                                 int64_t cap, int *__restrict__ counts) {
  __shared__ float t[kTY + 2][kTX + 2];
  const int map = blockIdx.z;
  const float *g = maps[map];
  const int64_t HW = (int64_t)H * W;
  const int tiles_x = (W + kTX - 1) / kTX;
  const int s = blockIdx.y;
  const int ty0 = (blockIdx.x / tiles_x) * kTY, tx0 = (blockIdx.x % tiles_x) * kTX;
  const float *gs = g + (int64_t)s * HW;
  for (int i = threadIdx.x; i < (kTY + 2) * (kTX + 2); i += blockDim.x) {
    const int yy = ty0 - 1 + i / (kTX + 2), xx = tx0 - 1 + i % (kTX + 2);
    // outside the grid: -inf never beats the centre (no strict neighbour test)
    t[i / (kTX + 2)][i % (kTX + 2)] =
        (yy >= 0 && yy < H && xx >= 0 && xx < W) ? __ldg(gs + (int64_t)yy * W + xx) : -INFINITY;
  }
  __syncthreads();
  const int ly = threadIdx.x / kTX, lx = threadIdx.x % kTX;
  const int y = ty0 + ly, x = tx0 + lx;
  bool lm = false;
  unsigned long long key = 0ull;
  if (y < H && x < W) {
    const float v = t[ly + 1][lx + 1];
    lm = !(t[ly][lx] > v) && !(t[ly][lx + 1] > v) && !(t[ly][lx + 2] > v) &&
         !(t[ly + 1][lx] > v) && !(t[ly + 1][lx + 2] > v) && !(t[ly + 2][lx] > v) &&
         !(t[ly + 2][lx + 1] > v) && !(t[ly + 2][lx + 2] > v);
    const int64_t i = (int64_t)s * HW + (int64_t)y * W + x;
    if (lm && s > 0) lm = g[i - HW] < v;
    if (lm && s < S - 1) lm = g[i + HW] < v;
    if (lm) {
      const uint32_t e = (uint32_t)((int64_t)s * HW + (int64_t)x * H + y);
      key = ((unsigned long long)ukey(v) << 32) | (unsigned long long)(0xFFFFFFFFu - e);
      if (key == 0ull) lm = false;  // NaN: never ranked (reference comparisons are false)
    }
  }
  const unsigned mask = __ballot_sync(0xFFFFFFFFu, lm);
  if (mask) {
    const int lane = threadIdx.x & 31;
    int pos0 = 0;
    if (lane == __ffs(mask) - 1) pos0 = atomicAdd(&counts[map], __popc(mask));
    pos0 = __shfl_sync(0xFFFFFFFFu, pos0, __ffs(mask) - 1);
    if (lm) {
      const int64_t p = pos0 + __popc(mask & ((1u << lane) - 1u));
      if (p < cap) keys[(int64_t)map * cap + p] = key;
    }
  }
}

// Bitonic sort of kChunk keys in shared memory, descending.
__device__ void bitonic_desc(unsigned long long *a) {
  for (int k = 2; k <= kChunk; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < kChunk; t += blockDim.x) {
        const int l = t ^ j;
        if (l > t) {
          const bool up = (t & k) == 0;  // this half sorts descending
          const unsigned long long x = a[t], y = a[l];
          if (up ? (x < y) : (x > y)) {
            a[t] = y;
            a[l] = x;
          }
        }
      }
      __syncthreads();
    }
}

// One level: chunk c of map m (its first n_in[m] keys are valid) -> its top
// k keys, sorted, zero-padded to exactly k, at out[m][c*k ...].
__global__ void __launch_bounds__(kThreads) k_lm_level(const unsigned long long *__restrict__ in,
                                                       const int *__restrict__ n_in,
                                                       int64_t in_cap,
                                                       unsigned long long *__restrict__ out,
                                                       int *__restrict__ n_out, int64_t out_cap,
                                                       int k) {
  __shared__ unsigned long long a[kChunk];
  const int map = blockIdx.y;
  const int64_t n = min((int64_t)n_in[map], in_cap);
  const int64_t start = (int64_t)blockIdx.x * kChunk;
  if (blockIdx.x == 0 && threadIdx.x == 0) n_out[map] = (int)(((n + kChunk - 1) / kChunk) * k);
  if (start >= n) return;
  const int m = (int)min((int64_t)kChunk, n - start);
  for (int t = threadIdx.x; t < kChunk; t += blockDim.x)
    a[t] = t < m ? in[(int64_t)map * in_cap + start + t] : 0ull;
  __syncthreads();
  bitonic_desc(a);
  unsigned long long *o = out + (int64_t)map * out_cap + (int64_t)blockIdx.x * k;
  for (int t = threadIdx.x; t < k; t += blockDim.x) o[t] = a[t];
}

// Final: at most kChunk keys left.  With total maxima <= k the reference
// lists them in enumeration order, else the k largest by value.
__global__ void __launch_bounds__(kThreads) k_lm_final(const unsigned long long *__restrict__ in,
                                                       const int *__restrict__ n_in,
                                                       int64_t in_cap,
                                                       const int *__restrict__ total, int k,
                                                       int S, int H, int W,
                                                       float *__restrict__ hyps,
                                                       int *__restrict__ n_hyps) {
  __shared__ unsigned long long a[kChunk];
  const int map = blockIdx.x;
  const int64_t n = min((int64_t)n_in[map], min(in_cap, (int64_t)kChunk));
  const int tot = total[map];
  for (int t = threadIdx.x; t < kChunk; t += blockDim.x)
    a[t] = t < n ? in[(int64_t)map * in_cap + t] : 0ull;
  __syncthreads();
  bitonic_desc(a);
  const int keep = tot < k ? tot : k;
  if (tot <= k) {
    // enumeration order: ascending index == descending low word
    for (int t = threadIdx.x; t < kChunk; t += blockDim.x)
      a[t] = t < keep ? ((a[t] << 32) | (a[t] >> 32)) : 0ull;
    __syncthreads();
    bitonic_desc(a);
    for (int t = threadIdx.x; t < kChunk; t += blockDim.x)
      if (t < keep) a[t] = (a[t] << 32) | (a[t] >> 32);
    __syncthreads();
  }
  const int64_t HW = (int64_t)H * W;
  float *o = hyps + (int64_t)map * k * 4;
  for (int t = threadIdx.x; t < keep; t += blockDim.x) {
    const unsigned long long key = a[t];
    const uint32_t e = 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFu);
    const int s = (int)(e / HW);
    const int64_t rem = e - (int64_t)s * HW;
    const int x = (int)(rem / H), y = (int)(rem - (int64_t)x * H);
    o[4 * t + 0] = (float)s;
    o[4 * t + 1] = (float)x;
    o[4 * t + 2] = (float)y;
    o[4 * t + 3] = ukey_decode((uint32_t)(key >> 32));
  }
  if (threadIdx.x == 0) n_hyps[map] = keep;
}

}  // namespace

// Scratch layout shared by the size query and the launcher: level sizes,
// the candidate keys, then one key buffer per selection level.
struct LmLayout {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  }
};

int local_max_kernels(int64_t cells, int k) {
  int n = 2;  // candidates + final
  int64_t cap = cells;
  while (cap > kChunk) {
    cap = ((cap + kChunk - 1) / kChunk) * k;
    ++n;
  }
  return n;
}

size_t local_max_scratch_bytes(int n_maps, int64_t cells, int k) {
  LmLayout L;
  L.take((size_t)n_maps * 3 * sizeof(int));
  L.take((size_t)n_maps * (size_t)cells * 8);
  int64_t cap = cells;
  while (cap > kChunk) {
    cap = ((cap + kChunk - 1) / kChunk) * k;
    L.take((size_t)n_maps * (size_t)cap * 8);
  }
  return L.off;
}

cudaError_t launch_local_max(const float *const *maps, int n_maps, int S, int H, int W, int k,
                             void *scratch, float *hyps, int *n_hyps, cudaStream_t s,
                             int *n_kernels) {
  if (k < 1 || k > kChunk / 2) return cudaErrorInvalidValue;
  const int64_t cells = (int64_t)S * H * W;
  char *base = static_cast<char *>(scratch);
  LmLayout L;
  int *counts = reinterpret_cast<int *>(base + L.take((size_t)n_maps * 3 * sizeof(int)));
  int *total = counts;                 // candidates per map (level-0 size)
  int *cnt_a = counts + n_maps;        // ping-pong level sizes
  int *cnt_b = counts + 2 * n_maps;
  unsigned long long *keys =
      reinterpret_cast<unsigned long long *>(base + L.take((size_t)n_maps * cells * 8));
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * 3 * n_maps, s);
  if (e != cudaSuccess) return e;
  const int tiles = ((H + kTY - 1) / kTY) * ((W + kTX - 1) / kTX);
  k_lm_cand<<<dim3((unsigned)tiles, (unsigned)S, (unsigned)n_maps), kTY * kTX, 0, s>>>(
      maps, S, H, W, keys, cells, total);
  int nk = 1;
  const unsigned long long *cur = keys;
  const int *cur_n = total;
  int64_t cur_cap = cells;
  int *next_n = cnt_a;
  while (cur_cap > kChunk) {
    const int64_t chunks = (cur_cap + kChunk - 1) / kChunk;
    const int64_t out_cap = chunks * k;
    unsigned long long *out =
        reinterpret_cast<unsigned long long *>(base + L.take((size_t)n_maps * out_cap * 8));
    k_lm_level<<<dim3((unsigned)chunks, (unsigned)n_maps), kThreads, 0, s>>>(cur, cur_n, cur_cap, out,
                                                                           next_n, out_cap, k);
    ++nk;
    cur = out;
    cur_n = next_n;
    next_n = (next_n == cnt_a) ? cnt_b : cnt_a;
    cur_cap = out_cap;
  }
  k_lm_final<<<(unsigned)n_maps, kThreads, 0, s>>>(cur, cur_n, cur_cap, total, k, S, H, W, hyps,
                                                   n_hyps);
  ++nk;
  if (n_kernels) *n_kernels = nk;
  return cudaGetLastError();
}

}  // namespace pa
