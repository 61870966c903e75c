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
// "larger value, then earlier in enumeration" and keys are unique.  A radix
// select over 8-bit digits finds the max_n-th largest key; the keys at or
// above its bin (at most kChunk) are gathered, sorted in shared memory and
// ordered by key (more than max_n maxima) or by enumeration index (at most
// max_n maxima).
#include "pa_internal.cuh"

namespace pa {
namespace {

constexpr int kChunk = 4096;
constexpr int kThreads = 1024;

// Candidates: a warp owns a block of kLmRows rows x 30 columns and walks all
// S slices of it.  Lane l holds column x0 - 1 + l (lanes 0 and 31 are the
// halo columns), so the left/right neighbours are lane shuffles; the rows
// above and below are neighbouring registers.  Slices s - 1, s, s + 1 are in
// registers while slice s + 2 is loaded, so every cell is read once and the
// loads of the next slice are in flight while the current one is tested.
// Cells outside the grid read -inf, which never beats the centre.
constexpr int kLmRows = 8;             // output rows per warp
constexpr int kLmCols = 30;            // output columns per warp
constexpr int kLmWarps = 8;
constexpr int kLmR = kLmRows + 2;      // rows held per slice (with halo)
constexpr int kLmBuf = 256;            // keys buffered per warp before a global append

__device__ __forceinline__ void lm_load_slice(float (&v)[kLmR], const float *gs, int ya, int H,
                                              int W, int x, bool on) {
#pragma unroll
  for (int j = 0; j < kLmR; ++j) {
    const int y = ya - 1 + j;
    v[j] = (on && y >= 0 && y < H && x >= 0 && x < W) ? __ldg(gs + (int64_t)y * W + x) : -INFINITY;
  }
}

__global__ void __launch_bounds__(32 * kLmWarps, 3) k_lm_cand(const float *const *__restrict__ maps,
                                                           int S, int H, int W,
                                                           unsigned long long *__restrict__ keys,
                                                           int64_t cap, int *__restrict__ counts) {
  __shared__ unsigned long long kbuf[kLmWarps][kLmBuf];
  const int map = blockIdx.z;
  const float *g = maps[map];
  const int64_t HW = (int64_t)H * W;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long *buf = kbuf[warp];
  int nbuf = 0;  // warp-uniform
  unsigned long long *dst = keys + (int64_t)map * cap;
  // one global reservation for the warp's buffered keys, coalesced writes
  auto flush = [&]() {
    int base = 0;
    if (lane == 0) base = atomicAdd(&counts[map], nbuf);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    __syncwarp();
    for (int i = lane; i < nbuf; i += 32)
      if ((int64_t)base + i < cap) dst[(int64_t)base + i] = buf[i];
    __syncwarp();
    nbuf = 0;
  };
  const int x0 = blockIdx.x * kLmCols;
  const int x = x0 - 1 + lane;
  const int ya = (blockIdx.y * kLmWarps + warp) * kLmRows;
  if (ya >= H) return;  // whole warp; no block-level synchronisation below
  const bool out_lane = lane >= 1 && lane <= kLmCols && x < W;
  float A[kLmR], B[kLmR], C[kLmR], D[kLmR];
#pragma unroll
  for (int j = 0; j < kLmR; ++j) A[j] = -INFINITY;
  lm_load_slice(B, g, ya, H, W, x, true);
  lm_load_slice(C, g + HW, ya, H, W, x, S > 1);
  for (int s = 0; s < S; ++s) {
    lm_load_slice(D, g + (int64_t)(s + 2) * HW, ya, H, W, x, s + 2 < S);
    // "no neighbour is greater" against row maxima: fmaxf skips NaN
    // neighbours, which never compare greater, so the test is unchanged
    float ml[kLmR], mh[kLmR];  // max of left/right; of left/centre/right
#pragma unroll
    for (int j = 0; j < kLmR; ++j) {
      ml[j] = fmaxf(__shfl_up_sync(0xFFFFFFFFu, B[j], 1), __shfl_down_sync(0xFFFFFFFFu, B[j], 1));
      mh[j] = fmaxf(ml[j], B[j]);
    }
#pragma unroll
    for (int j = 1; j <= kLmRows; ++j) {
      const int y = ya - 1 + j;
      const float v = B[j];
      bool lm = out_lane && y < H && !(mh[j - 1] > v) && !(ml[j] > v) && !(mh[j + 1] > v);
      if (s > 0) lm = lm && A[j] < v;
      if (s < S - 1) lm = lm && C[j] < v;
      unsigned long long key = 0ull;
      if (lm) {
        const uint32_t e = (uint32_t)((int64_t)s * HW + (int64_t)x * H + y);
        key = ((unsigned long long)ukey(v) << 32) | (unsigned long long)(0xFFFFFFFFu - e);
        if (key == 0ull) lm = false;
      }
      const unsigned mask = __ballot_sync(0xFFFFFFFFu, lm);
      if (mask) {
        if (nbuf + 32 > kLmBuf) flush();
        if (lm) buf[nbuf + __popc(mask & ((1u << lane) - 1u))] = key;
        nbuf += __popc(mask);
      }
    }
#pragma unroll
    for (int j = 0; j < kLmR; ++j) {
      A[j] = B[j];
      B[j] = C[j];
      C[j] = D[j];
    }
  }
  __syncwarp();
  if (nbuf) flush();
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

// Radix select of the top k keys of every map (keys are unique: the low
// word is the enumeration index).  Pass d looks at bits [56 - 8d, 64 - 8d) of
// the keys that share the bits above with `prefix`: every CTA histograms a
// stride of the keys, and the last CTA to finish (arrival counter; no CTA
// waits on another) picks the bin b that holds the k_rem-th largest key.
// Keys in higher bins are selected for sure; the pass ends the search when
// bin b holds at most `room` keys, so the final gather collects at most
// k + room <= kChunk keys.
struct LmState {
  unsigned long long prefix;
  int k_rem;
  int shift;    // bits below the decided prefix when done
  int done;     // 1: prefix decided; 2: every candidate is selected
  int arrive;
  int pad[2];
};

__global__ void __launch_bounds__(256) k_lm_radix(const unsigned long long *__restrict__ keys,
                                                  const int *__restrict__ counts, int64_t cap,
                                                  int pass, int room,
                                                  unsigned int *__restrict__ hist,
                                                  LmState *__restrict__ state) {
  __shared__ unsigned int h[256];
  __shared__ int last;
  const int map = blockIdx.y;
  LmState *st = state + map;
  if (st->done) return;  // decided by an earlier pass (uniform for the CTA)
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int64_t n = min((int64_t)counts[map], cap);
  const int shift = 56 - 8 * pass;
  const unsigned long long prefix = st->prefix;
  const unsigned long long *k = keys + (int64_t)map * cap;
  // lanes that fall into the same bin add once (bins are crowded: most
  // marginal values share their top bits)
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_pad = (n + 31) / 32 * 32;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += stride) {
    int bin = -1;
    if (i < n) {
      const unsigned long long key = k[i];
      if (pass == 0 || (key >> (shift + 8)) == (prefix >> (shift + 8)))
        bin = (int)((key >> shift) & 255u);
    }
    const unsigned same = __match_any_sync(0xFFFFFFFFu, bin);
    if (bin >= 0 && (threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&h[bin], (unsigned)__popc(same));
  }
  __syncthreads();
  unsigned int *g = hist + (int64_t)map * 256;
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&g[i], h[i]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(&st->arrive, 1) == (int)gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last CTA: read the complete histogram (through L2) and decide
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    h[i] = __ldcg(&g[i]);
    g[i] = 0;  // ready for the next pass
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    st->arrive = 0;
    const int k_rem = st->k_rem;
    unsigned int total = 0;
    for (int b = 0; b < 256; ++b) total += h[b];
    if (pass == 0 && total <= (unsigned)k_rem) {
      st->done = 2;
    } else {
      unsigned int cum = 0;
      int b = 255;
      for (; b > 0; --b) {
        if (cum + h[b] >= (unsigned)k_rem) break;
        cum += h[b];
      }
      st->prefix = prefix | ((unsigned long long)b << shift);
      st->k_rem = k_rem - (int)cum;
      if (h[b] <= (unsigned)room || shift == 0) {
        st->shift = shift;
        st->done = 1;
      }
    }
  }
}

__global__ void k_lm_init(LmState *__restrict__ state, int n_maps, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_maps) return;
  LmState s;
  s.prefix = 0ull;
  s.k_rem = k;
  s.shift = 0;
  s.done = 0;
  s.arrive = 0;
  s.pad[0] = s.pad[1] = 0;
  state[i] = s;
}

// Final: gather the selected keys (all candidates, or those at or above the
// decided prefix: at most kChunk), sort them, keep k.  With total maxima
// <= k the reference lists them in enumeration order, else the k largest by
// value.
__global__ void __launch_bounds__(kThreads) k_lm_final(const unsigned long long *__restrict__ keys,
                                                       const int *__restrict__ counts, int64_t cap,
                                                       const LmState *__restrict__ state, int k,
                                                       int S, int H, int W,
                                                       float *__restrict__ hyps,
                                                       int *__restrict__ n_hyps) {
  __shared__ unsigned long long a[kChunk];
  __shared__ int na;
  const int map = blockIdx.x;
  const int64_t n = min((int64_t)counts[map], cap);
  const LmState st = state[map];
  for (int t = threadIdx.x; t < kChunk; t += blockDim.x) a[t] = 0ull;
  if (threadIdx.x == 0) na = 0;
  __syncthreads();
  const unsigned long long *src = keys + (int64_t)map * cap;
  const bool all = st.done == 2;
  const unsigned long long lo = st.prefix;  // keys >= lo: selected or in the boundary bin
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long key = src[i];
    if (all || (key >> st.shift) >= (lo >> st.shift)) {
      const int p = atomicAdd(&na, 1);
      if (p < kChunk) a[p] = key;
    }
  }
  __syncthreads();
  bitonic_desc(a);
  const int tot = (int)n;
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

constexpr int kRadixPasses = 8;  // 8-bit digits of the 64-bit keys
constexpr int kRadixCtas = 8;    // CTAs per map in a histogram pass

int local_max_kernels(int64_t cells, int k, int stages) {
  (void)cells;
  (void)k;
  return ((stages & LM_CAND) ? 2 : 0) + ((stages & LM_SELECT) ? kRadixPasses : 0) +
         ((stages & LM_FINAL) ? 1 : 0);  // init + candidates, passes, final
}

size_t local_max_scratch_bytes(int n_maps, int64_t cells, int k) {
  (void)k;
  LmLayout L;
  L.take((size_t)n_maps * sizeof(int));
  L.take((size_t)n_maps * sizeof(LmState));
  L.take((size_t)n_maps * 256 * sizeof(unsigned int));
  L.take((size_t)n_maps * (size_t)cells * 8);
  return L.off;
}

cudaError_t launch_local_max(const float *const *maps, int n_maps, int S, int H, int W, int k,
                             void *scratch, float *hyps, int *n_hyps, cudaStream_t s,
                             int *n_kernels, int stages) {
  if (k < 1 || k > kChunk / 2) return cudaErrorInvalidValue;
  const int64_t cells = (int64_t)S * H * W;
  if (cells > 0xFFFFFFFFll) return cudaErrorInvalidValue;  // 32-bit enumeration index
  char *base = static_cast<char *>(scratch);
  LmLayout L;
  int *counts = reinterpret_cast<int *>(base + L.take((size_t)n_maps * sizeof(int)));
  LmState *state = reinterpret_cast<LmState *>(base + L.take((size_t)n_maps * sizeof(LmState)));
  unsigned int *hist =
      reinterpret_cast<unsigned int *>(base + L.take((size_t)n_maps * 256 * sizeof(unsigned int)));
  unsigned long long *keys =
      reinterpret_cast<unsigned long long *>(base + L.take((size_t)n_maps * cells * 8));
  if (n_maps > 65535) return cudaErrorInvalidValue;
  int nk = 0;
  if (stages & LM_CAND) {
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * n_maps, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, sizeof(unsigned int) * 256 * n_maps, s);
    if (e != cudaSuccess) return e;
    k_lm_init<<<(n_maps + 127) / 128, 128, 0, s>>>(state, n_maps, k);
    const int rows_per_cta = kLmWarps * kLmRows;
    k_lm_cand<<<dim3((unsigned)((W + kLmCols - 1) / kLmCols),
                     (unsigned)((H + rows_per_cta - 1) / rows_per_cta), (unsigned)n_maps),
                32 * kLmWarps, 0, s>>>(maps, S, H, W, keys, cells, counts);
    nk += 2;
  }
  if (stages & LM_SELECT) {
    const int room = kChunk - k;
    for (int pass = 0; pass < kRadixPasses; ++pass)
      k_lm_radix<<<dim3(kRadixCtas, (unsigned)n_maps), 256, 0, s>>>(keys, counts, cells, pass,
                                                                     room, hist, state);
    nk += kRadixPasses;
  }
  if (stages & LM_FINAL) {
    k_lm_final<<<(unsigned)n_maps, kThreads, 0, s>>>(keys, counts, cells, state, k, S, H, W, hyps,
                                                     n_hyps);
    nk += 1;
  }
  if (n_kernels) *n_kernels = nk;
  return cudaGetLastError();
}

}  // namespace pa
