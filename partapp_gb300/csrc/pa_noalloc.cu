// pa_noalloc.cu -- computeRotJointMarginal for callers that cannot allocate.
//
// Some hosts of this library may not allocate device memory on the call
// path: an application that reserved the whole device for its own memory
// pool at start-up (so cudaMalloc fails or would exceed its budget), or a
// latency-critical loop that must not hit cudaMalloc/cudaFree, which can
// synchronise the device.  pa_rot_joint_marginal_noalloc serves them: it runs
// the same message kernels as pa_rot_joint_marginal, but every intermediate
// (the exp-domain row-filtered map, the shift tables, the filter taps, the
// message descriptor, the max/error words) lives in one file-scope device
// array, g_noalloc_scratch, whose size is fixed at compile time.  Every GPU
// that loads the library holds that array until the process exits.
//
// Limits: R * H * W <= PA_NOALLOC_MAX_CELLS (2^21 cells, e.g. 24 x 240 x 320),
// 2 <= R <= 64, H + W <= 4096, at most 1024 spatial taps per axis
// (sigma <= 170 px).  Larger sizes return PA_ERR_NOMEM and touch nothing.
//
// The array is shared by every call on a device and keeps the contents of
// the last call; the max and error words are cleared at the start of each
// call, every other region is fully rewritten.  Calls whose GPU work
// overlaps (two streams, or two host threads) race on the array.
//
// Set-up: every call, with the target device current, looks up the array's
// device address with cudaGetSymbolAddress (the symbol's name is a host-side
// stand-in, not a device address).  The lookup allocates nothing; doing it on
// every call keeps the address right after a cudaDeviceReset, which gives the
// device a new primary context and the array a new address.  The first call
// on a device may load the library's module onto it, so make that first call
// before any stream capture.
#include <cstring>

#include "pa_internal.cuh"

namespace pa {
namespace {

constexpr size_t al256(size_t v) { return (v + 255) / 256 * 256; }

constexpr int kNoAllocMaxR = kMaxRot;             // 64 rotations
constexpr int kNoAllocMaxWH = 4096;               // H + W
constexpr int kNoAllocMaxTaps = 1024;             // per spatial axis
constexpr size_t kOffDesc = 0;
constexpr size_t kOffRtaps = al256(kOffDesc + sizeof(MsgDesc));
constexpr size_t kOffXtaps = al256(kOffRtaps + kNoAllocMaxR * sizeof(float));
constexpr size_t kOffYtaps = al256(kOffXtaps + kNoAllocMaxTaps * sizeof(float));
constexpr size_t kOffShifts = al256(kOffYtaps + kNoAllocMaxTaps * sizeof(float));
constexpr size_t kOffSdesc = al256(kOffShifts + 4 * kNoAllocMaxR * sizeof(double));
constexpr size_t kOffWords = al256(kOffSdesc + 4 * kNoAllocMaxR * sizeof(int4));
constexpr size_t kOffTables = al256(kOffWords + 2 * sizeof(int));
constexpr size_t kOffE2 = al256(kOffTables + (size_t)2 * kNoAllocMaxR * kNoAllocMaxWH * sizeof(int16_t));
constexpr size_t kScratchBytes = al256(kOffE2 + (size_t)PA_NOALLOC_MAX_CELLS * sizeof(float));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch on the current device.
cudaError_t scratch_address(unsigned char **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<unsigned char *>(p);
  return cudaSuccess;
}

// True for device (or managed) memory of the current device: a buffer on
// another GPU would be reached through peer addressing, or fault.
bool on_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace
}  // namespace pa

using namespace pa;

extern "C" pa_status pa_rot_joint_marginal_noalloc(const pa_exp_param *ep, const float *child,
                                                   float *parent, int R, int H, int W,
                                                   const double *offset_c,
                                                   const double *offset_p, const double *C,
                                                   double rot_mean, double rot_sigma,
                                                   double scale, void *stream) {
  if (!ep || !child || !parent || !offset_c || !offset_p || !C) return PA_ERR_INVALID;
  if (R != ep->num_rotation_steps || R < 2 || H < 1 || W < 1 ||
      !(ep->max_part_rotation > ep->min_part_rotation))
    return PA_ERR_INVALID;
  if (R > kNoAllocMaxR || H + W > kNoAllocMaxWH ||
      (int64_t)R * H * W > (int64_t)PA_NOALLOC_MAX_CELLS)
    return PA_ERR_NOMEM;  // beyond the fixed scratch array
  if (C[1] != 0 || C[2] != 0) return PA_ERR_UNSUPPORTED;
  if (!(C[0] > 0 && C[3] > 0)) return PA_ERR_INVALID;
  if (!on_device(child) || !on_device(parent)) return PA_ERR_INVALID;

  MsgParams mp;
  msg_params(ep, scale, offset_c, offset_p, C, rot_mean, rot_sigma, H, W, false, mp);
  if (mp.xlen > kNoAllocMaxTaps || mp.ylen > kNoAllocMaxTaps) return PA_ERR_NOMEM;

  unsigned char *base = nullptr;
  if (scratch_address(&base) != cudaSuccess) {
    cudaGetLastError();
    return PA_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t N = (int64_t)R * H * W;
  int *slot = reinterpret_cast<int *>(base + kOffWords);
  int *err = slot + 1;
  int16_t *tables = reinterpret_cast<int16_t *>(base + kOffTables);
  int4 *sdesc = reinterpret_cast<int4 *>(base + kOffSdesc);
  double *shifts = reinterpret_cast<double *>(base + kOffShifts);

  MsgDesc d;
  std::memset(&d, 0, sizeof d);
  d.in = child;
  d.in_max = slot;
  d.e2 = reinterpret_cast<float *>(base + kOffE2);
  d.tx_in = tables;
  d.ty_in = tables + (size_t)R * W;
  d.tx_out = tables + (size_t)R * (W + H);
  d.ty_out = tables + (size_t)R * (W + H) + (size_t)R * W;
  d.sdesc = sdesc;
  d.rtaps = reinterpret_cast<const float *>(base + kOffRtaps);
  d.xtaps = reinterpret_cast<const float *>(base + kOffXtaps);
  d.ytaps = reinterpret_cast<const float *>(base + kOffYtaps);
  d.kidx = mp.kidx;
  d.rlen = mp.rlen;
  d.xlen = mp.xlen;
  d.ylen = mp.ylen;
  d.mode = EPI_STORE;
  d.dst0 = parent;

  // parameters: copies from host memory into the array (no allocation)
  cudaError_t e = cudaSuccess;
  auto put = [&](size_t off, const void *src, size_t bytes) {
    if (e == cudaSuccess && bytes)
      e = cudaMemcpyAsync(base + off, src, bytes, cudaMemcpyHostToDevice, s);
  };
  put(kOffDesc, &d, sizeof d);
  put(kOffRtaps, mp.rtaps.data(), mp.rtaps.size() * sizeof(float));
  put(kOffXtaps, mp.xtaps.data(), mp.xtaps.size() * sizeof(float));
  put(kOffYtaps, mp.ytaps.data(), mp.ytaps.size() * sizeof(float));
  put(kOffShifts, mp.shifts.data(), mp.shifts.size() * sizeof(double));
  const MsgDesc *dd = reinterpret_cast<const MsgDesc *>(base + kOffDesc);
  // words that must start at their identity: max = -inf, error = 0
  if (e == cudaSuccess) e = launch_fill_int(slot, kFkeyNegInf, 1, s);
  if (e == cudaSuccess) e = launch_fill_int(err, 0, 1, s);
  if (e == cudaSuccess) e = launch_map_max(child, N, slot, s);
  if (e == cudaSuccess) e = launch_shift_tables(shifts, 1, R, H, W, tables, sdesc, s);
  if (e == cudaSuccess) e = launch_msg_rows(dd, 1, R, H, W, (mp.xlen - 1) / 2, err, s);
  if (e == cudaSuccess) e = launch_msg_cols(dd, 1, R, H, W, (mp.ylen - 1) / 2, err, s);
  int errflag = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&errflag, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PA_ERR_CUDA;
  }
  if (errflag & 1) return PA_ERR_NUMERIC;
  if (errflag) return PA_ERR_UNSUPPORTED;
  return PA_OK;
}
