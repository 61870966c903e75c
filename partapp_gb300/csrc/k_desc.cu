// k_desc.cu -- SHAPEv5 shape-context descriptor grid on GB300.
//
// Replaces computeDescriptorGrid (libPartDetect/partdetect_aux.cpp:77-190)
// with the SHAPEv5 descriptor of libKMA2 (ShapeDescriptor.cpp:168-261): for
// every position of a rotated grid, a 21 x 21 patch is resampled from the
// image (ImageContent::interpolate), normalised to mean 128 / deviation 50
// (normalize, FeatureDescriptor.cpp:80-113), its central-difference
// gradients (dX2 / dY2) go through Canny (EdgeDetector.cpp:74-147) and the
// edge magnitudes are binned by log-polar position and orientation into 96
// values, normalised, clipped at 0.2, renormalised and quantised.
//
// One warp owns one grid position; its patch and the intermediate maps live
// in the warp's slice of shared memory.  Elementwise steps run on all 32
// lanes; the steps whose float sums or scan order define the result (the
// patch mean and variance, the Canny raster scan with its label
// propagation, the histogram accumulation, the vector norms) run on lane 0
// in the reference's order, so the arithmetic matches the reference's
// operation for operation.  No multiply-add is fused: every product that
// feeds a sum goes through an explicitly rounded intrinsic, in float or in
// double as the reference's expression types dictate.  The one library
// function whose result can differ in the last bit from the host's is
// atan2f (gradient orientation).
#include <climits>

#include <cstddef>

#include "pa_internal.cuh"

namespace pa {
namespace {

constexpr int kP = 21;          // PATCH_SIZE, libKMA2/descriptor/feature.h:25
constexpr int kPP = kP * kP;
constexpr int kHalf = kP / 2;
constexpr int kShape = 96;      // SrSize * ScSize * SOriSize (3 * 4 * 8), ShapeDescriptor.h:35-37
constexpr int kSr = 3, kSc = 4, kSOri = 8;
constexpr float kMaxIndexVal = 0.2f;  // ShapeDescriptor.h:38
constexpr float kColor = 255.f;       // EdgeDetector.cpp:79
constexpr float kLower = 5.f, kHigher = 15.f;  // cannyEdges(dx, dy, grad, edge, 5, 15)
constexpr double kPi = 3.14159265358979323846;
constexpr float kPiAbove = 3.14159274101257324f;  // the float nearest pi, above it
constexpr int kDescWarps = 4;   // grid positions (one per warp) per CTA
constexpr int kChunk = 88;      // histogram samples per increment batch (fits patch + grad)

struct WarpScratch {
  float patch[kPP];          // patch, then Canny candidates, then histogram increments
  float grad[kPP];           // (adjacent to patch: the increments use both)
  float ori[kPP], edge[kPP];
  float vec[kShape];
  float sum, fac;
  unsigned short tmp[kPP + 1];  // weak-edge labels, then the histogram sample list
  unsigned char cor[kPP + 1];   // connected-to-strong flag per label
  unsigned char state[kPP];     // 0 none, 1 strong edge, 2 weak edge candidate
};

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// ---------------------------------------------------------------------------
// FP32 fast path of the double-typed interpolation expressions.  The
// reference evaluates them in double and rounds once to float.  Here they are
// evaluated in float-float arithmetic (Knuth's TwoSum and the FMA form of
// Dekker's TwoProduct are exact), and the float result is used only when it
// is certain to be the double result's rounding: with all terms
// non-negative, the double evaluation is within 6 * 2^-53 and the float-float
// one within about 2^-43 of the exact value, so every value within 2^-40 of
// the float-float sum rounds to the same float unless that sum lies within
// 2^-40 (relative) of a rounding midpoint.  Those rare cases, and operands
// outside the analysed ranges, take the double path, so the bits never change.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bv = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
}

__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// r = the float nearest to hi + lo, when every value within 2^-40 (relative)
// of hi + lo rounds to it.
__device__ __forceinline__ bool certified_round(float hi, float lo, float &r) {
  float sr, e;
  two_sum(hi, lo, sr, e);  // sr = fl(hi + lo), sr + e = hi + lo
  if (!(sr >= 0x1p-100f && sr < 0x1p100f)) {
    if (hi == 0.f && lo == 0.f) {
      r = 0.f;
      return true;
    }
    return false;
  }
  const unsigned b = __float_as_uint(sr);
  const float up = __fsub_rn(__uint_as_float(b + 1u), sr);  // spacing above sr (exact)
  const float dn = __fsub_rn(sr, __uint_as_float(b - 1u));  // spacing below sr (exact)
  const float half = 0.5f * (e >= 0.f ? up : dn);
  if (__fadd_ru(fabsf(e), sr * 0x1p-40f) < half) {
    r = sr;
    return true;
  }
  return false;
}

// (1 - t) * a + fl(t * b) for t in [0, 1), a, b >= 0: hi + lo within about
// 2^-46 of the exact value (1 - t is exact as oh + ol).
__device__ __forceinline__ void ff_lerp(float t, float a, float b, float &hi, float &lo) {
  float oh, ol, ph, pl, sh, sl;
  two_sum(1.f, -t, oh, ol);
  two_prod(oh, a, ph, pl);
  two_sum(ph, __fmul_rn(t, b), sh, sl);
  hi = sh;
  lo = __fadd_rn(__fadd_rn(sl, pl), __fmul_rn(ol, a));
}

__device__ __forceinline__ bool lerp_ok(float t, float a, float b) {
  return t >= 0.f && t < 1.f && a >= 0.f && b >= 0.f;
}

// (1 - dy) * ((1 - dx) * a + dx * b) + dy * ((1 - dx) * c + dx * d) with the
// reference's types: 1.0 - d in double, dx * b a float product.
__device__ __forceinline__ float bilinear4(float dx, float dy, float a, float b, float c, float d) {
  if (lerp_ok(dx, a, b) && lerp_ok(dy, c, d) && dy >= 0.f && c >= 0.f) {
    float t1h, t1l, t2h, t2l, oh, ol, uh, ul, vh, vl, wh, wl, r;
    ff_lerp(dx, a, b, t1h, t1l);
    ff_lerp(dx, c, d, t2h, t2l);
    two_sum(1.f, -dy, oh, ol);
    two_prod(oh, t1h, uh, ul);
    two_prod(dy, t2h, vh, vl);
    const float cross = __fadd_rn(__fadd_rn(__fmul_rn(oh, t1l), __fmul_rn(ol, t1h)),
                                  __fmul_rn(dy, t2l));
    two_sum(uh, vh, wh, wl);
    if (certified_round(wh, __fadd_rn(__fadd_rn(__fadd_rn(wl, ul), vl), cross), r)) return r;
  }
  const double omdx = dsub(1.0, (double)dx), omdy = dsub(1.0, (double)dy);
  const double t1 = dadd(dmul(omdx, (double)a), (double)fmul(dx, b));
  const double t2 = dadd(dmul(omdx, (double)c), (double)fmul(dx, d));
  return __double2float_rn(dadd(dmul(omdy, t1), dmul((double)dy, t2)));
}

// (1.0 - t) * a + t * b, 1.0 - t in double, t * b a float product.
__device__ __forceinline__ float lerp1(float t, float a, float b) {
  if (lerp_ok(t, a, b)) {
    float hi, lo, r;
    ff_lerp(t, a, b, hi, lo);
    if (certified_round(hi, lo, r)) return r;
  }
  return __double2float_rn(dadd(dmul(dsub(1.0, (double)t), (double)a), (double)fmul(t, b)));
}

// ImageContent::getValue (ImageContent.cpp:29-50) on a 21 x 21 map.
__device__ float get_value(const float *g, float x, float y) {
  const unsigned ix = (unsigned)(long long)floorf(x);
  const unsigned iy = (unsigned)(long long)floorf(y);
  const float dx = fsub(x, (float)ix), dy = fsub(y, (float)iy);
  const unsigned n = kP - 1;
  if (ix < n && iy < n)
    return bilinear4(dx, dy, g[iy * kP + ix], g[iy * kP + ix + 1], g[(iy + 1) * kP + ix],
                     g[(iy + 1) * kP + ix + 1]);
  // (1.0 - dy) * a + dy * b: the second product is a float one
  if (ix == n && iy < n) return lerp1(dy, g[iy * kP + ix], g[(iy + 1) * kP + ix]);
  if (iy == n && ix < n) return lerp1(dx, g[iy * kP + ix], g[iy * kP + ix + 1]);
  if (iy == n && ix == n) return g[iy * kP + ix];
  return 0.f;
}

// r = the float nearest to hi + lo when every value within m_abs of hi + lo
// rounds to it (for sums that may cancel, with an absolute error bound).
__device__ __forceinline__ bool certified_round_abs(float hi, float lo, float m_abs, float &r) {
  float sr, e;
  two_sum(hi, lo, sr, e);
  if (!(sr >= 0x1p-100f && sr < 0x1p100f)) return false;
  const unsigned b = __float_as_uint(sr);
  const float up = __fsub_rn(__uint_as_float(b + 1u), sr);
  const float dn = __fsub_rn(sr, __uint_as_float(b - 1u));
  const float half = 0.5f * (e >= 0.f ? up : dn);
  if (__fadd_ru(fabsf(e), m_abs) < half) {
    r = sr;
    return true;
  }
  return false;
}

// fl_f(fl_d(m * (1.0 - f))) for m >= 0, f in [0, 1): m * (1 - f) = m * oh + m * ol
// with the first product exact, within about 2^-46; the double path otherwise.
__device__ __forceinline__ float weight_om(float m, float f) {
  if (m >= 0.f && f >= 0.f && f < 1.f) {
    float oh, ol, ph, pl, r;
    two_sum(1.f, -f, oh, ol);
    two_prod(m, oh, ph, pl);
    if (certified_round(ph, __fadd_rn(pl, __fmul_rn(m, ol)), r)) return r;
  }
  return __double2float_rn(dmul((double)m, dsub(1.0, (double)f)));
}

// pi (the double constant) as a float pair: kPiAbove + kPiLo = pi within 2^-49.
constexpr float kPiLo = (float)(kPi - (double)kPiAbove);

// fl_f(fl_d((double)x / pi)) for x >= 0: q0 = fl(x / kPiAbove), the remainder
// x - q0 * kPiAbove exact by FMA, the correction q1 within about 2^-46.
__device__ __forceinline__ float div_pi(float x) {
  if (x >= 0.f && x < 0x1p100f) {
    const float q0 = __fdiv_rn(x, kPiAbove);
    const float rem = __fmaf_rn(-q0, kPiAbove, x);
    const float q1 = __fdiv_rn(__fmaf_rn(-q0, kPiLo, rem), kPiAbove);
    float r;
    if (certified_round(q0, q1, r)) return r;
  }
  return __double2float_rn(__ddiv_rn((double)x, kPi));
}

// fl_f(fl_d((double)o + pi)) for o in [-pi, 0): o + kPiAbove exact as a pair, plus
// kPiLo, within 2^-44 absolute (the sum can cancel).
__device__ __forceinline__ float add_pi(float o) {
  float sh, sl, r;
  two_sum(o, kPiAbove, sh, sl);
  if (certified_round_abs(sh, __fadd_rn(sl, kPiLo), 0x1p-44f, r)) return r;
  return __double2float_rn(dadd((double)o, kPi));
}

// (int)(v >= 0 ? (double)v : (double)v - 1.0): truncating v - 1 for v < 0
// is ceil(v) - 1, exact in float.
__device__ __forceinline__ int index_below(float v) {
  return v >= 0.0f ? (int)v : (int)ceilf(v) - 1;
}

// KMAPlaceInLogPolIndex (ShapeDescriptor.cpp:71-121), orientation modulo pi:
// the up to 8 (bin, weight) increments of one sample, in the reference's
// r -> c -> orientation order (bin 255: no increment).
__device__ void place_entries(float mag, float ori, float rx, float cx, uint8_t *bins, float *ws) {
  const float oval = div_pi(fmul((float)kSOri, ori));
  const int ri = index_below(rx), ci = index_below(cx), oi = index_below(oval);
  const float rfrac = fsub(rx, (float)ri), cfrac = fsub(cx, (float)ci), ofrac = fsub(oval, (float)oi);
  for (int r = 0; r < 2; ++r) {
    const int rindex = ri + r;
    const bool rok = rindex >= 0 && rindex < kSr;
    // m * frac: the double product of two floats is exact, so its rounding
    // is the float product
    const float rweight = r == 0 ? weight_om(mag, rfrac) : fmul(mag, rfrac);
    for (int c = 0; c < 2; ++c) {
      int cindex = ci + c;
      if (cindex >= kSc) cindex = 0;
      const bool cok = rok && cindex >= 0 && cindex < kSc;
      const float cweight = c == 0 ? weight_om(rweight, cfrac) : fmul(rweight, cfrac);
      const int rcindex = (rindex * kSc + cindex) << 3;
      for (int ort = 0; ort < 2; ++ort) {
        int oindex = oi + ort;
        if (oindex >= kSOri) oindex = 0;
        const int e = (r * 2 + c) * 2 + ort;
        bins[e] = cok ? (uint8_t)(rcindex + oindex) : (uint8_t)255;
        ws[e] = cok ? (ort == 0 ? weight_om(cweight, ofrac) : fmul(cweight, ofrac)) : 0.f;
      }
    }
  }
}

// KMANormalizeVect (ShapeDescriptor.cpp:26-39), lane 0.  fac = 1.0 / sqrt(sqlen)
// divides in double and rounds to float; a quotient of two floats rounded
// first to 53 and then to 24 bits equals the correctly rounded float quotient
// (53 >= 2 * 24 + 2, Figueroa's double-rounding bound), so the float division
// gives the same bits without the FP64 pipe.
__device__ void normalize_vect(float *v) {
  float sqlen = 0.f;
  for (int i = 0; i < kShape; ++i) sqlen = fadd(sqlen, fmul(v[i], v[i]));
  const float fac = __fdiv_rn(1.f, __fsqrt_rn(sqlen));
  for (int i = 0; i < kShape; ++i) v[i] = fmul(v[i], fac);
}

__global__ void __launch_bounds__(32 * kDescWarps, 5) k_shape_grid(
    const float *__restrict__ img, int h, int w, DescGrid g, const DescTables *__restrict__ tabs,
    float *__restrict__ cells, uint8_t *__restrict__ valid) {
  extern __shared__ __align__(16) unsigned char dsm[];
  DescTables &T = *reinterpret_cast<DescTables *>(dsm);
  WarpScratch *scratch = reinterpret_cast<WarpScratch *>(dsm + sizeof(DescTables));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  {
    const int *src = reinterpret_cast<const int *>(tabs);
    int *dst = reinterpret_cast<int *>(&T);
    for (int i = threadIdx.x; i < (int)(sizeof(DescTables) / 4); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int64_t cell = (int64_t)blockIdx.x * kDescWarps + warp;
  if (cell >= (int64_t)g.nx * g.ny) return;  // uniform for the warp; no block barrier follows
  WarpScratch &S = scratch[warp];
  const int iy = (int)(cell / g.nx), ix = (int)(cell - (int64_t)iy * g.nx);
  float *out = cells + cell * kShape;

  // grid -> image position (partdetect_aux.cpp:133-142) and the inside test
  const double x2 = dadd(g.min_x, dmul((double)ix, g.step));
  const double y2 = dadd(g.min_y, dmul((double)iy, g.step));
  const double px = dadd(dadd(0.0, dmul(x2, g.ax0)), dmul(y2, g.ay0));
  const double py = dadd(dadd(0.0, dmul(x2, g.ax1)), dmul(y2, g.ay1));
  bool skip = !(px >= g.lo_x && px <= g.hi_x && py >= g.lo_y && py <= g.hi_y);
  if (!skip && g.mask) {
    // detection_mask[imgpos(1)][imgpos(0)] == 0 (partdetect_aux.cpp:132-138);
    // px, py >= 1 here, so the truncation is a floor
    const long long mx = (long long)px - g.mask_ox, my = (long long)py - g.mask_oy;
    skip = mx < 0 || my < 0 || mx >= g.mask_w || my >= g.mask_h ||
           g.mask[my * g.mask_w + mx] == 0.f;
  }
  if (skip) {
    for (int k = lane; k < kShape; k += 32) out[k] = 0.f;
    if (lane == 0) valid[cell] = 0;
    return;
  }
  const float mx = __double2float_rn(px), my = __double2float_rn(py);

  // (1) ImageContent::interpolate (ImageContent.cpp:658-727)
  const int xim = w - 1, yim = h - 1;
  for (int k = lane; k < kPP; k += 32) {
    const int j = k / kP - kHalf, i = k - (k / kP) * kP - kHalf;
    const float pxf = fadd(fadd(mx, fmul((float)i, g.v0x)), fmul((float)j, g.v0y));
    const float pyf = fadd(fadd(my, fmul((float)i, g.v1x)), fmul((float)j, g.v1y));
    const int ax = (int)floorf(pxf), ay = (int)floorf(pyf);
    const float dx = fsub(pxf, (float)ax), dy = fsub(pyf, (float)ay);
    float v = 0.f;
    if (ax >= 0 && ay >= 0 && ax < xim && ay < yim) {
      const float *r0 = img + (int64_t)ay * w + ax;
      v = bilinear4(dx, dy, r0[0], r0[1], r0[w], r0[w + 1]);
    } else if (ax < 0 && ay < 0) {
      v = img[0];
    } else if (ax >= xim && ay >= yim) {
      v = img[(int64_t)yim * w + xim];
    } else if (ax < 0 && ay > yim) {
      v = img[(int64_t)yim * w];
    } else if (ax >= xim && ay < 0) {
      v = img[xim];
    } else if (ax > xim && ay >= 0) {
      v = img[(int64_t)ay * w + xim];
    } else if (ax >= 0 && ay < 0) {
      v = img[ax];
    } else if (ax >= 0 && ay >= yim) {
      v = img[(int64_t)yim * w + ax];
    } else if (ax < 0 && ay >= 0) {
      v = img[(int64_t)ay * w];
    } else if (ax >= xim && ay >= 0) {
      v = img[(int64_t)ay * w + xim];
    }
    S.patch[k] = v;
  }
  __syncwarp();

  // (2) normalize: mean and deviation over the mask, in the reference's order
  if (lane == 0) {
    float sum = 0.f, gsum = 0.f;
    for (int k = 0; k < kPP; ++k)
      if (T.mask[k] > 0) {
        sum = fadd(sum, S.patch[k]);
        gsum = fadd(gsum, 1.f);
      }
    sum = __fdiv_rn(sum, gsum);
    float var = 0.f;
    for (int k = 0; k < kPP; ++k)
      if (T.mask[k] > 0) {
        const float d = fsub(sum, S.patch[k]);
        var = fadd(var, fmul(d, d));
      }
    var = __fsqrt_rn(__fdiv_rn(var, gsum));
    S.sum = sum;
    S.fac = __fdiv_rn(50.f, var);  // 50.0 / var in double, rounded: the same bits (see normalize_vect)
  }
  __syncwarp();
  {
    const float sum = S.sum, fac = S.fac;
    for (int k = lane; k < kPP; k += 32) {
      float v = fadd(128.f, fmul(fac, fsub(S.patch[k], sum)));
      if (v > 255) v = 255;
      if (v < 0) v = 0;
      S.patch[k] = v;
    }
  }
  __syncwarp();

  // (3) dX2 / dY2 (gauss_iir.cpp:1182-1225), magnitude and orientation
  for (int k = lane; k < kPP; k += 32) {
    const int y = k / kP, x = k - y * kP;
    const bool in = y >= 1 && y < kP - 1 && x >= 1 && x < kP - 1;
    const float ddx = in ? fsub(S.patch[k + 1], S.patch[k - 1]) : 0.f;
    const float ddy = in ? fsub(S.patch[k + kP], S.patch[k - kP]) : 0.f;
    S.grad[k] = __fsqrt_rn(fadd(fmul(ddx, ddx), fmul(ddy, ddy)));
    S.ori[k] = atan2f(ddy, ddx);
    S.edge[k] = 0.f;
    S.tmp[k] = 0;
  }
  __syncwarp();

  // (4) Canny: non-maximum suppression on all lanes ...
  for (int k = lane; k < kPP; k += 32) {
    const int j = k / kP, i = k - j * kP;
    unsigned char st = 0;
    if (j >= 1 && j < kP - 2 && i >= 1 && i < kP - 2) {
      const float gv = S.grad[k];
      if (!(gv < kLower)) {
        // dX2 / dY2 at an interior pixel, recomputed (the patch is still intact)
        const float ux = fsub(S.patch[k + 1], S.patch[k - 1]);
        const float uy = fsub(S.patch[k + kP], S.patch[k - kP]);
        const float qx = __fdiv_rn(ux, gv), qy = __fdiv_rn(uy, gv);
        const float g1 = get_value(S.grad, fadd((float)i, qx), fadd((float)j, qy));
        const float g2 = get_value(S.grad, fsub((float)i, qx), fsub((float)j, qy));
        if (gv <= g1 || gv <= g2) st = 0;
        else if (gv > kHigher) st = 1;
        else if (gv > kLower) st = 2;
      }
    }
    S.state[k] = st;
  }
  __syncwarp();
  // ... the candidates in raster order (the patch buffer is free by now) ...
  short *cand = reinterpret_cast<short *>(S.patch);
  int ncand = 0;
  for (int base = 0; base < kPP; base += 32) {
    const int k = base + lane;
    const bool c = k < kPP && S.state[k] != 0;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, c);
    if (c) cand[ncand + __popc(m & ((1u << lane) - 1u))] = (short)k;
    ncand += __popc(m);
  }
  __syncwarp();
  // ... and the raster scan with its order-dependent promotion and labels on lane 0
  if (lane == 0) {
    int nb = 1;  // the reference counts labels in a float; they stay below 2^24
    S.cor[0] = 0;
    for (int n = 0; n < ncand; ++n) {
      const int k = cand[n];
      {
        const unsigned char st = S.state[k];
        if (st == 1) {
          S.edge[k] = kColor;
        } else if (S.edge[k - kP - 1] == kColor || S.edge[k - kP] == kColor ||
                   S.edge[k - kP + 1] == kColor || S.edge[k - 1] == kColor) {
          S.edge[k] = kColor;
        } else if (S.tmp[k - kP - 1] > 0) {
          S.tmp[k] = S.tmp[k - kP - 1];
        } else if (S.tmp[k - kP] > 0) {
          S.tmp[k] = S.tmp[k - kP];
        } else if (S.tmp[k - kP + 1] > 0) {
          S.tmp[k] = S.tmp[k - kP + 1];
        } else if (S.tmp[k - 1] > 0) {
          S.tmp[k] = S.tmp[k - 1];
        } else if (S.tmp[k + 1] > 0) {
          S.tmp[k] = S.tmp[k + 1];
        } else {
          S.tmp[k] = (unsigned short)nb;
          S.cor[nb] = 0;
          ++nb;
        }
      }
    }
  }
  __syncwarp();
  // labels touching an edge pixel (8-neighbourhood) join it
  for (int k = lane; k < kPP; k += 32) {
    const int j = k / kP, i = k - j * kP;
    if (j < 1 || j > kP - 2 || i < 1 || i > kP - 2) continue;
    const float *e = S.edge;
    if (e[k - kP - 1] == kColor || e[k - kP] == kColor || e[k - kP + 1] == kColor ||
        e[k - 1] == kColor || e[k + 1] == kColor || e[k + kP - 1] == kColor ||
        e[k + kP] == kColor || e[k + kP + 1] == kColor)
      S.cor[S.tmp[k]] = 1;
  }
  __syncwarp();
  for (int k = lane; k < kPP; k += 32) {
    const int j = k / kP, i = k - j * kP;
    if (j < 1 || j > kP - 2 || i < 1 || i > kP - 2) continue;
    if (S.tmp[k] > 0 && S.cor[S.tmp[k]] == 1) S.edge[k] = kColor;
  }
  __syncwarp();
  for (int k = lane; k < kPP; k += 32) S.edge[k] = S.edge[k] > 0 ? S.grad[k] : 0.f;
  __syncwarp();

  // (5) log-polar histogram (KMAcomputeShape's sampling loop, :209-237, and
  // KMAAddLogPolSample, :126-164).  The loop visits (i, j) with i outer, so
  // its pixel k = (10 + i) * 21 + (10 + j) runs through 0..440 in order.
  // (a) the samples that add to the histogram, in that order
  short *list = reinterpret_cast<short *>(S.tmp);  // the labels are no longer needed
  int nlist = 0;
  for (int base = 0; base < kPP; base += 32) {
    const int k = base + lane;
    bool c = false;
    if (k < kPP) {
      const int i = k / kP - kHalf, j = k - (k / kP) * kP - kHalf;
      // (double)edge < 1e-10  <=>  edge < the smallest float >= 1e-10
      c = T.inrange[(kHalf + j) * kP + (kHalf + i)] && !(S.edge[k] < __uint_as_float(0x2EDBE6FFu));
    }
    const unsigned m = __ballot_sync(0xFFFFFFFFu, c);
    if (c) list[nlist + __popc(m & ((1u << lane) - 1u))] = (short)k;
    nlist += __popc(m);
  }
  __syncwarp();
  // (b) chunks of samples: all lanes compute the increments (double
  // arithmetic), then lane b accumulates bins b, b + 32, b + 64 in the
  // reference's order
  // patch and grad (adjacent, free now): kChunk * 8 weights, then the bins
  static_assert(offsetof(WarpScratch, grad) == offsetof(WarpScratch, patch) + kPP * sizeof(float),
                "grad must follow patch");
  static_assert(kChunk * 8 * (sizeof(float) + 1) <= 2 * kPP * sizeof(float),
                "histogram increments must fit in patch + grad");
  float *ws = reinterpret_cast<float *>(reinterpret_cast<char *>(&S) + offsetof(WarpScratch, patch));
  uint8_t *bins = reinterpret_cast<uint8_t *>(ws + kChunk * 8);
  float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f;
  for (int c0 = 0; c0 < nlist; c0 += kChunk) {
    const int nc = min(kChunk, nlist - c0);
    for (int n = lane; n < nc; n += 32) {
      const int k = list[c0 + n];
      const int i = k / kP - kHalf, j = k - (k / kP) * kP - kHalf;
      const int t = (kHalf + j) * kP + (kHalf + i);  // patch_lcpos(iradius + j, iradius + i)
      const float mag = fmul(T.mask[k], S.edge[k]);
      float o = fsub(S.ori[k], 0.f);
      // (double)o > pi  <=>  o >= the float just above pi
      while (o >= kPiAbove) o = __double2float_rn(dsub((double)o, kPi));
      while (o < 0.f) o = add_pi(o);
      place_entries(mag, o, T.lr[t], T.lc[t], bins + n * 8, ws + n * 8);
    }
    __syncwarp();
    for (int e = 0; e < nc * 8; ++e) {
      const int b = bins[e];
      const float wv = ws[e];
      if (b == lane) acc0 = fadd(acc0, wv);
      else if (b == lane + 32) acc1 = fadd(acc1, wv);
      else if (b == lane + 64) acc2 = fadd(acc2, wv);
    }
    __syncwarp();
  }
  S.vec[lane] = acc0;
  S.vec[lane + 32] = acc1;
  S.vec[lane + 64] = acc2;
  __syncwarp();
  // (c) norms and quantisation, lane 0
  if (lane == 0) {
    normalize_vect(S.vec);
    bool changed = false;
    for (int i = 0; i < kShape; ++i)
      if (S.vec[i] > kMaxIndexVal) {
        S.vec[i] = kMaxIndexVal;
        changed = true;
      }
    if (changed) normalize_vect(S.vec);
    for (int i = 0; i < kShape; ++i) {
      // (int)(512.0 * v): scaling by a power of two is exact in float too.  A
      // NaN (a patch without edges) truncates to INT_MIN on x86-64, where the
      // reference runs
      const float s = fmul(512.f, S.vec[i]);
      const int iv = (s != s) ? INT_MIN : (int)s;
      S.vec[i] = (float)((255 < iv) ? 255 : iv);
    }
  }
  __syncwarp();
  for (int k = lane; k < kShape; k += 32) out[k] = S.vec[k];
  if (lane == 0) valid[cell] = 1;
}

// One line of the recursive Gaussian (horizontal() / vertical(),
// libKMA2/gauss_iir/gauss_iir.cpp:197-420): causal pass y+ stored in out,
// anticausal pass y- folded in as out = (y+ + y-) * scale.  Every sum runs
// left to right over rounded float products, as the reference's
// expressions do.
__device__ void iir_line(const float *__restrict__ in, float *__restrict__ out, int n, int st,
                         const IirCoefs &cf) {
  const float *c = cf.c;
  const float n00p = c[0], n11p = c[1], n22p = c[2], n33p = c[3], n11m = c[4], n22m = c[5],
              n33m = c[6], n44m = c[7], d11p = c[8], d22p = c[9], d33p = c[10], d44p = c[11],
              d11m = c[12], d22m = c[13], d33m = c[14], d44m = c[15], scale = c[16];
  auto I = [&](int k) { return in[(int64_t)k * st]; };
  // a0*b0 + a1*b1 + a2*b2 + a3*b3 - e0*f0 - e1*f1 - e2*f2 - e3*f3
  auto rec = [&](float a0, float b0, float a1, float b1, float a2, float b2, float a3, float b3,
                 float e0, float f0, float e1, float f1, float e2, float f2, float e3, float f3) {
    float t = fmul(a0, b0);
    t = fadd(t, fmul(a1, b1));
    t = fadd(t, fmul(a2, b2));
    t = fadd(t, fmul(a3, b3));
    t = fsub(t, fmul(e0, f0));
    t = fsub(t, fmul(e1, f1));
    t = fsub(t, fmul(e2, f2));
    return fsub(t, fmul(e3, f3));
  };
  const float np = fadd(fadd(fadd(n00p, n11p), n22p), n33p);
  const float dp = fadd(fadd(fadd(d11p, d22p), d33p), d44p);
  float z = __fdiv_rn(np, fadd(1.f, dp));
  const float i0 = I(0), i1 = I(1), i2 = I(2), i3 = I(3);
  float p0 = fmul(z, i0);
  float p1 = fsub(fadd(fadd(fadd(fmul(n00p, i1), fmul(n11p, i0)), fmul(n22p, i0)), fmul(n33p, i0)),
                  fmul(dp, p0));
  float p2 = rec(n00p, i2, n11p, i1, n22p, i0, n33p, i0, d11p, p1, d22p, p0, d33p, p0, d44p, p0);
  float p3 = rec(n00p, i3, n11p, i2, n22p, i1, n33p, i0, d11p, p2, d22p, p1, d33p, p0, d44p, p0);
  out[0] = p0;
  out[(int64_t)st] = p1;
  out[(int64_t)2 * st] = p2;
  out[(int64_t)3 * st] = p3;
  float a1 = i3, a2 = i2, a3 = i1;          // I(k-1), I(k-2), I(k-3)
  float q1 = p3, q2 = p2, q3 = p1, q4 = p0;  // p(k-1) .. p(k-4)
  for (int k = 4; k < n; ++k) {
    const float ik = I(k);
    const float pk = rec(n00p, ik, n11p, a1, n22p, a2, n33p, a3, d11p, q1, d22p, q2, d33p, q3,
                         d44p, q4);
    out[(int64_t)k * st] = pk;
    a3 = a2;
    a2 = a1;
    a1 = ik;
    q4 = q3;
    q3 = q2;
    q2 = q1;
    q1 = pk;
  }
  const float nm = fadd(fadd(fadd(n11m, n22m), n33m), n44m);
  const float dm = fadd(fadd(fadd(d11m, d22m), d33m), d44m);
  z = __fdiv_rn(nm, fadd(1.f, dm));
  const int e = n - 1;
  const float ie = I(e), ie1 = I(e - 1), ie2 = I(e - 2), ie3 = I(e - 3);
  const float m0 = fmul(z, ie);
  const float m1 = fsub(fmul(nm, ie), fmul(dm, m0));
  const float m2 = rec(n11m, ie1, n22m, ie, n33m, ie, n44m, ie, d11m, m1, d22m, m0, d33m, m0, d44m, m0);
  const float m3 = rec(n11m, ie2, n22m, ie1, n33m, ie, n44m, ie, d11m, m2, d22m, m1, d33m, m0, d44m, m0);
  auto fold = [&](int k, float m) {
    float *o = out + (int64_t)k * st;
    *o = fmul(fadd(*o, m), scale);
  };
  fold(e, m0);
  fold(e - 1, m1);
  fold(e - 2, m2);
  fold(e - 3, m3);
  float b1 = ie3, b2 = ie2, b3 = ie1, b4 = ie;  // I(k+1) .. I(k+4)
  float r1 = m3, r2 = m2, r3 = m1, r4 = m0;     // m(k+1) .. m(k+4)
  for (int k = n - 5; k >= 0; --k) {
    const float mk = rec(n11m, b1, n22m, b2, n33m, b3, n44m, b4, d11m, r1, d22m, r2, d33m, r3,
                         d44m, r4);
    fold(k, mk);
    b4 = b3;
    b3 = b2;
    b2 = b1;
    b1 = I(k);
    r4 = r3;
    r3 = r2;
    r2 = r1;
    r1 = mk;
  }
}

// smooth(): the recursive Gaussian along y (one thread per column) ...
__global__ void k_iir_y(const float *__restrict__ in, float *__restrict__ out, int h, int w,
                        IirCoefs cf) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x < w) iir_line(in + x, out + x, h, w, cf);
}
// ... then along x (one thread per row)
__global__ void k_iir_x(const float *__restrict__ in, float *__restrict__ out, int h, int w,
                        IirCoefs cf) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y < h) iir_line(in + (int64_t)y * w, out + (int64_t)y * w, w, 1, cf);
}

// add_image_border2: copy, then mirrored columns left/right (rows b..b+h-1),
// then mirrored rows top/bottom over the full width (from the padded image).
__global__ void k_border_cols(const float *__restrict__ in, int h, int w, int b,
                              float *__restrict__ out) {
  const int W2 = w + 2 * b;
  const int64_t n = (int64_t)h * W2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int yy = (int)(i / W2), xx = (int)(i - (int64_t)yy * W2);
    int sx;
    if (xx < b) sx = b - 1 - xx;                // out[.][bidx-1] = in[.][b-bidx]
    else if (xx < b + w) sx = xx - b;
    else sx = w - 1 - (xx - b - w);             // out[.][b+w+bidx-1] = in[.][w-bidx]
    out[(int64_t)(b + yy) * W2 + xx] = in[(int64_t)yy * w + sx];
  }
}
__global__ void k_border_rows(int h, int w, int b, float *__restrict__ out) {
  const int W2 = w + 2 * b;
  const int64_t n = (int64_t)2 * b * W2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / W2), xx = (int)(i - (int64_t)k * W2);
    if (k < b) {  // top row bidx - 1 = k from row 2b - 1 - k (inside the copied band)
      out[(int64_t)k * W2 + xx] = out[(int64_t)(2 * b - 1 - k) * W2 + xx];
    } else {      // bottom row b + h + j from row b + h - 1 - j
      const int j = k - b;
      out[(int64_t)(b + h + j) * W2 + xx] = out[(int64_t)(b + h - 1 - j) * W2 + xx];
    }
  }
}

__global__ void k_grid_bbox(const float *const *__restrict__ grids, int ny, int nx,
                            int4 *__restrict__ bbox) {
  __shared__ int mnx, mny, mxx, mxy;
  if (threadIdx.x == 0) {
    mnx = nx;
    mny = ny;
    mxx = -1;
    mxy = -1;
  }
  __syncthreads();
  const float *g = grids[blockIdx.x];
  int a = nx, c = ny, d = -1, e = -1;
  for (int i = threadIdx.x; i < nx * ny; i += blockDim.x)
    if (g[i] != kNoClassValue) {
      const int y = i / nx, x = i - y * nx;
      a = min(a, x);
      c = min(c, y);
      d = max(d, x);
      e = max(e, y);
    }
  atomicMin(&mnx, a);
  atomicMin(&mny, c);
  atomicMax(&mxx, d);
  atomicMax(&mxy, e);
  __syncthreads();
  if (threadIdx.x == 0) bbox[blockIdx.x] = make_int4(mnx, mny, mxx, mxy);
}

}  // namespace

cudaError_t launch_mirror_border(const float *in, int h, int w, int b, float *out,
                                 cudaStream_t s) {
  if (b < 0 || b >= w || b >= h) return cudaErrorInvalidValue;
  k_border_cols<<<608, 256, 0, s>>>(in, h, w, b, out);
  if (b > 0) k_border_rows<<<152, 256, 0, s>>>(h, w, b, out);
  return cudaGetLastError();
}

cudaError_t launch_grid_bbox(const float *const *grids, int n, int ny, int nx, int4 *bbox,
                             cudaStream_t s) {
  if (n < 1) return cudaSuccess;
  k_grid_bbox<<<(unsigned)n, 1024, 0, s>>>(grids, ny, nx, bbox);
  return cudaGetLastError();
}

cudaError_t launch_smooth(const float *in, float *tmp, float *out, int h, int w,
                          const IirCoefs &cf, cudaStream_t s) {
  if (h < 5 || w < 5) return cudaErrorInvalidValue;
  k_iir_y<<<(unsigned)((w + 127) / 128), 128, 0, s>>>(in, tmp, h, w, cf);
  k_iir_x<<<(unsigned)((h + 127) / 128), 128, 0, s>>>(tmp, out, h, w, cf);
  return cudaGetLastError();
}

size_t desc_smem_bytes() { return sizeof(DescTables) + kDescWarps * sizeof(WarpScratch); }

cudaError_t launch_shape_grid(const float *img, int h, int w, const DescGrid &g,
                              const DescTables *tabs, float *cells, uint8_t *valid,
                              cudaStream_t s) {
  const int64_t n = (int64_t)g.nx * g.ny;
  if (n <= 0) return cudaSuccess;
  const size_t smem = desc_smem_bytes();
  cudaFuncSetAttribute(k_shape_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_shape_grid<<<(unsigned)((n + kDescWarps - 1) / kDescWarps), 32 * kDescWarps, smem, s>>>(
      img, h, w, g, tabs, cells, valid);
  return cudaGetLastError();
}

}  // namespace pa
