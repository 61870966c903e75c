/* desc.cpp -- CPU restatement of the SHAPEv5 shape-context descriptor grid
 * (libPartDetect/partdetect_aux.cpp:77-190, computeDescriptorGrid, and the
 * libKMA2 code it calls).  TEST INFRASTRUCTURE ONLY, like oracle.cpp: the
 * checker for the GPU descriptor kernels, never part of the product path.
 *
 * Every floating-point expression keeps the reference's types (float where
 * the reference stores float, double where a double literal or a double
 * variable promotes it) and its evaluation order; the file is compiled with
 * -ffp-contract=off so no multiply-add is fused.  The one place where the
 * reference depends on its platform is the conversion of a NaN to int
 * ((int)(512.0 * NaN) in KMAcomputeShape, reached by patches without edges):
 * x86-64, where the reference runs, yields INT_MIN; this file writes INT_MIN
 * explicitly so that x86 and Arm hosts agree. */
#include "oracle.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

/* libKMA2/descriptor/feature.h:25, ShapeDescriptor.h:35-38 */
constexpr int kPatch = 21;
constexpr int kSr = 3, kSc = 4, kSOri = 8;
constexpr int kShape = kSr * kSc * kSOri;
constexpr float kMaxIndexVal = 0.2f;
/* libKMA2/gauss_iir/gauss_iir.h:21 */
constexpr double kM2Pi = 6.2831853072;

/* num_scale_steps, scale_from_index(0) and rot_from_index
 * (libPartApp/partapp_aux.hpp:45-58, 86-129), as oracle.cpp states them */
int n_scales_desc(const orc_exp *e) { return e->num_scale_steps > 1 ? e->num_scale_steps : 1; }
double scale_value(const orc_exp *e, int idx) {
  if (e->min_object_scale == e->max_object_scale) return e->min_object_scale;
  const double step = ((double)e->max_object_scale - e->min_object_scale) / n_scales_desc(e);
  return e->min_object_scale + step * (0.5 + idx);
}
double rot_value(const orc_exp *e, int idx) {
  if (e->min_part_rotation == e->max_part_rotation) return e->min_part_rotation;
  const double step = ((double)e->max_part_rotation - e->min_part_rotation) /
                      (double)(unsigned)e->num_rotation_steps;
  return e->min_part_rotation + step * (0.5 + idx);
}

struct Img {  /* DARY: fel[row][col], x() = columns, y() = rows */
  int w, h;
  const float *p;
  float at(int r, int c) const { return p[(size_t)r * w + c]; }
};

/* ImageContent::interpolate, ImageContent/ImageContent.cpp:658-727: a
 * kPatch x kPatch patch sampled around (m_x, m_y) along the two axes, with
 * the reference's clamping of samples that fall off the image. */
void interpolate(const Img &in, float m_x, float m_y, float vec0x, float vec0y, float vec1x,
                 float vec1y, float *patch) {
  const int half = kPatch >> 1;
  const int xim = in.w - 1, yim = in.h - 1;
  for (int j = -half; j <= half; ++j)
    for (int i = -half; i <= half; ++i) {
      const float px = m_x + i * vec0x + j * vec0y;
      const float py = m_y + i * vec1x + j * vec1y;
      const int ax = (int)std::floor(px), ay = (int)std::floor(py);
      const float dx = px - ax, dy = py - ay;
      float &o = patch[(j + half) * kPatch + (i + half)];
      if (ax >= 0 && ay >= 0 && ax < xim && ay < yim) {
        o = (float)((1.0 - dy) * ((1.0 - dx) * in.at(ay, ax) + dx * in.at(ay, ax + 1)) +
                    dy * ((1.0 - dx) * in.at(ay + 1, ax) + dx * in.at(ay + 1, ax + 1)));
      } else if (ax < 0 && ay < 0) {
        o = in.at(0, 0);
      } else if (ax >= xim && ay >= yim) {
        o = in.at(yim, xim);
      } else if (ax < 0 && ay > yim) {
        o = in.at(yim, 0);
      } else if (ax >= xim && ay < 0) {
        o = in.at(0, xim);
      } else if (ax > xim && ay >= 0) {
        o = in.at(ay, xim);
      } else if (ax >= 0 && ay < 0) {
        o = in.at(0, ax);
      } else if (ax >= 0 && ay >= yim) {
        o = in.at(yim, ax);
      } else if (ax < 0 && ay >= 0) {
        o = in.at(ay, 0);
      } else if (ax >= xim && ay >= 0) {
        o = in.at(ay, xim);
      }
    }
}

/* ImageContent::getValue, ImageContent/ImageContent.cpp:29-50 */
float get_value(const float *g, int w, int h, float x, float y) {
  const unsigned ix = (unsigned)(long long)std::floor(x);
  const unsigned iy = (unsigned)(long long)std::floor(y);
  const float dx = x - ix, dy = y - iy;
  const unsigned xs = (unsigned)w, ys = (unsigned)h;
  auto at = [&](unsigned r, unsigned c) { return g[(size_t)r * w + c]; };
  float val = 0;
  if (ix < xs - 1 && iy < ys - 1) {
    val = (float)((1.0 - dy) * ((1.0 - dx) * at(iy, ix) + dx * at(iy, ix + 1)) +
                  dy * ((1.0 - dx) * at(iy + 1, ix) + dx * at(iy + 1, ix + 1)));
  } else if (ix == xs - 1 && iy < ys - 1) {
    val = (float)((1.0 - dy) * at(iy, ix) + dy * (at(iy + 1, ix)));
  } else if (iy == ys - 1 && ix < xs - 1) {
    val = (float)((1.0 - dx) * at(iy, ix) + dx * (at(iy, ix + 1)));
  } else if (iy == ys - 1 && ix == xs - 1) {
    val = at(iy, ix);
  }
  return val;
}

/* normalize, descriptor/FeatureDescriptor.cpp:80-113 */
void normalize_patch(float *img, const float *mask) {
  float sum = 0, gsum = 0;
  for (int j = 0; j < kPatch; ++j)
    for (int i = 0; i < kPatch; ++i)
      if (mask[j * kPatch + i] > 0) {
        sum += img[j * kPatch + i];
        gsum++;
      }
  sum = sum / gsum;
  float var = 0;
  for (int j = 0; j < kPatch; ++j)
    for (int i = 0; i < kPatch; ++i)
      if (mask[j * kPatch + i] > 0)
        var += (sum - img[j * kPatch + i]) * (sum - img[j * kPatch + i]);
  var = std::sqrt(var / gsum);
  const float fac = 50.0 / var;
  for (int k = 0; k < kPatch * kPatch; ++k) {
    img[k] = 128 + fac * (img[k] - sum);
    if (img[k] > 255) img[k] = 255;
    if (img[k] < 0) img[k] = 0;
  }
}

/* cannyEdges(dx, dy, grad, edge, lower, higher), descriptor/EdgeDetector.cpp:74-147:
 * non-maximum suppression along the gradient, strong edges above `higher`,
 * weak ones kept when connected to a strong one (raster-order labels). */
void canny(const float *dx, const float *dy, const float *grad, float *edge, float lower,
           float higher) {
  const int W = kPatch, H = kPatch;
  std::vector<float> tmp(W * H, 0.f);
  std::vector<int> cor{0};
  const float color = 255;
  float nb = 1;
  auto E = [&](int j, int i) -> float & { return edge[j * W + i]; };
  auto T = [&](int j, int i) -> float & { return tmp[j * W + i]; };
  for (int j = 1; j < H - 2; ++j)
    for (int i = 1; i < W - 2; ++i) {
      const float g = grad[j * W + i];
      if (g < lower) continue;
      const float ux = dx[j * W + i], uy = dy[j * W + i];
      const float x1 = i + ux / g, y1 = j + uy / g;
      const float x2 = i - ux / g, y2 = j - uy / g;
      const float g1 = get_value(grad, W, H, x1, y1);
      const float g2 = get_value(grad, W, H, x2, y2);
      if (g <= g1 || g <= g2) continue;
      if (g > higher) {
        E(j, i) = color;
      } else if (g > lower && (E(j - 1, i - 1) == color || E(j - 1, i) == color ||
                               E(j - 1, i + 1) == color || E(j, i - 1) == color)) {
        E(j, i) = color;
      } else if (g > lower) {
        if (T(j - 1, i - 1) > 0) T(j, i) = T(j - 1, i - 1);
        else if (T(j - 1, i) > 0) T(j, i) = T(j - 1, i);
        else if (T(j - 1, i + 1) > 0) T(j, i) = T(j - 1, i + 1);
        else if (T(j, i - 1) > 0) T(j, i) = T(j, i - 1);
        else if (T(j, i + 1) > 0) T(j, i) = T(j, i + 1);
        else {
          T(j, i) = nb;
          cor.push_back(0);
          nb++;
        }
      }
    }
  for (int j = H - 2; j > 0; --j)
    for (int i = W - 2; i > 0; --i)
      if (E(j - 1, i - 1) == color || E(j - 1, i) == color || E(j - 1, i + 1) == color ||
          E(j, i - 1) == color || E(j, i + 1) == color || E(j + 1, i - 1) == color ||
          E(j + 1, i) == color || E(j + 1, i + 1) == color)
        cor[(int)T(j, i)] = 1;
  for (int j = H - 2; j > 0; --j)
    for (int i = W - 2; i > 0; --i)
      if (T(j, i) > 0 && cor[(int)T(j, i)] == 1) E(j, i) = color;
  for (int k = 0; k < W * H; ++k) edge[k] = edge[k] > 0 ? grad[k] : 0;
}

/* KMANormalizeVect, ShapeDescriptor.cpp:26-39 */
void normalize_vect(float *v) {
  float sqlen = 0.0;
  for (int i = 0; i < kShape; ++i) sqlen += v[i] * v[i];
  const float fac = 1.0 / std::sqrt(sqlen);
  for (int i = 0; i < kShape; ++i) v[i] *= fac;
}

/* KMAPlaceInLogPolIndex, ShapeDescriptor.cpp:71-121 (orientation modulo pi) */
void place(float *index, float mag, float ori, float rx, float cx) {
  const float oval = kSOri * ori / (M_PI);
  const int ri = (int)((rx >= 0.0) ? rx : rx - 1.0);
  const int ci = (int)((cx >= 0.0) ? cx : cx - 1.0);
  const int oi = (int)((oval >= 0.0) ? oval : oval - 1.0);
  const float rfrac = rx - ri, cfrac = cx - ci, ofrac = oval - oi;
  for (int r = 0; r < 2; ++r) {
    const int rindex = ri + r;
    if (rindex >= 0 && rindex < kSr) {
      const float rweight = mag * ((r == 0) ? 1.0 - rfrac : rfrac);
      for (int c = 0; c < 2; ++c) {
        int cindex = ci + c;
        if (cindex >= kSc) cindex = 0;
        if (cindex >= 0 && cindex < kSc) {
          const float cweight = rweight * ((c == 0) ? 1.0 - cfrac : cfrac);
          const int rcindex = (rindex * kSc + cindex) << 3;
          for (int ort = 0; ort < 2; ++ort) {
            int oindex = oi + ort;
            if (oindex >= kSOri) oindex = 0;
            const float oweight = cweight * ((ort == 0) ? 1.0 - ofrac : ofrac);
            index[rcindex + oindex] += oweight;
          }
        }
      }
    }
  }
}

/* set_nii_and_dii + set_smooth_coefficients, gauss_iir.cpp:47-120: the
 * fourth-order recursive Gaussian (Deriche) of width sigma, in float. */
void smooth_coefficients(float sigma, float *coefs) {
  const float a0 = 1.68f, a1 = 3.735f, b0 = 1.783f, b1 = 1.723f, c0 = -0.6803f, c1 = -0.2598f,
              omega0 = 0.6318f, omega1 = 1.997f;
  coefs[0] = a0 + c0;
  coefs[1] = std::exp(-b1 / sigma) * (c1 * std::sin(omega1 / sigma) - (c0 + 2 * a0) * std::cos(omega1 / sigma)) +
             std::exp(-b0 / sigma) * (a1 * std::sin(omega0 / sigma) - (2 * c0 + a0) * std::cos(omega0 / sigma));
  coefs[2] = 2 * std::exp(-b0 / sigma - b1 / sigma) *
                 ((a0 + c0) * std::cos(omega1 / sigma) * std::cos(omega0 / sigma) -
                  std::cos(omega1 / sigma) * a1 * std::sin(omega0 / sigma) -
                  std::cos(omega0 / sigma) * c1 * std::sin(omega1 / sigma)) +
             c0 * std::exp(-2 * b0 / sigma) + a0 * std::exp(-2 * b1 / sigma);
  coefs[3] = std::exp(-b1 / sigma - 2 * b0 / sigma) * (c1 * std::sin(omega1 / sigma) - c0 * std::cos(omega1 / sigma)) +
             std::exp(-b0 / sigma - 2 * b1 / sigma) * (a1 * std::sin(omega0 / sigma) - a0 * std::cos(omega0 / sigma));
  coefs[8] = -2 * std::exp(-b1 / sigma) * std::cos(omega1 / sigma) - 2 * std::exp(-b0 / sigma) * std::cos(omega0 / sigma);
  coefs[9] = 4 * std::cos(omega1 / sigma) * std::cos(omega0 / sigma) * std::exp(-b0 / sigma - b1 / sigma) +
             std::exp(-2 * b1 / sigma) + std::exp(-2 * b0 / sigma);
  coefs[10] = -2 * std::cos(omega0 / sigma) * std::exp(-b0 / sigma - 2 * b1 / sigma) -
              2 * std::cos(omega1 / sigma) * std::exp(-b1 / sigma - 2 * b0 / sigma);
  coefs[11] = std::exp(-2 * b0 / sigma - 2 * b1 / sigma);
  coefs[12] = coefs[8];
  coefs[13] = coefs[9];
  coefs[14] = coefs[10];
  coefs[15] = coefs[11];
  coefs[4] = coefs[1] - coefs[8] * coefs[0];
  coefs[5] = coefs[2] - coefs[9] * coefs[0];
  coefs[6] = coefs[3] - coefs[10] * coefs[0];
  coefs[7] = -coefs[11] * coefs[0];
  coefs[16] = 1 / (std::sqrt(2 * 3.141) * sigma);
}

/* One recursive pass along a line of n samples at stride st (the body of
 * horizontal() / vertical(), gauss_iir.cpp:197-420): causal y+, anticausal
 * y-, out = (y+ + y-) * scale.  out may not alias in. */
void iir_line(const float *in, float *out, int n, int st, const float *c) {
  const float n00p = c[0], n11p = c[1], n22p = c[2], n33p = c[3], n11m = c[4], n22m = c[5],
              n33m = c[6], n44m = c[7], d11p = c[8], d22p = c[9], d33p = c[10], d44p = c[11],
              d11m = c[12], d22m = c[13], d33m = c[14], d44m = c[15], scale = c[16];
  auto I = [&](int k) { return in[(size_t)k * st]; };
  std::vector<float> p(n), m(n);
  const float np = n00p + n11p + n22p + n33p;
  const float dp = d11p + d22p + d33p + d44p;
  float z = np / (1 + dp);
  p[0] = z * I(0);
  p[1] = n00p * I(1) + n11p * I(0) + n22p * I(0) + n33p * I(0) - dp * p[0];
  p[2] = n00p * I(2) + n11p * I(1) + n22p * I(0) + n33p * I(0) - d11p * p[1] - d22p * p[0] -
         d33p * p[0] - d44p * p[0];
  p[3] = n00p * I(3) + n11p * I(2) + n22p * I(1) + n33p * I(0) - d11p * p[2] - d22p * p[1] -
         d33p * p[0] - d44p * p[0];
  for (int k = 4; k < n; ++k)
    p[k] = n00p * I(k) + n11p * I(k - 1) + n22p * I(k - 2) + n33p * I(k - 3) - d11p * p[k - 1] -
           d22p * p[k - 2] - d33p * p[k - 3] - d44p * p[k - 4];
  const float nm = n11m + n22m + n33m + n44m;
  const float dm = d11m + d22m + d33m + d44m;
  z = nm / (1 + dm);
  const int e = n - 1;
  m[e] = z * I(e);
  m[e - 1] = nm * I(e) - dm * m[e];
  m[e - 2] = n11m * I(e - 1) + n22m * I(e) + n33m * I(e) + n44m * I(e) - d11m * m[e - 1] -
             d22m * m[e] - d33m * m[e] - d44m * m[e];
  m[e - 3] = n11m * I(e - 2) + n22m * I(e - 1) + n33m * I(e) + n44m * I(e) - d11m * m[e - 2] -
             d22m * m[e - 1] - d33m * m[e] - d44m * m[e];
  for (int k = n - 5; k >= 0; --k)
    m[k] = n11m * I(k + 1) + n22m * I(k + 2) + n33m * I(k + 3) + n44m * I(k + 4) -
           d11m * m[k + 1] - d22m * m[k + 2] - d33m * m[k + 3] - d44m * m[k + 4];
  for (int k = 0; k < n; ++k) out[(size_t)k * st] = (p[k] + m[k]) * scale;
}

}  // namespace

extern "C" {

/* smooth(image_in, smooth_image, scale), gauss_iir.cpp:1391-1400: the
 * recursive Gaussian along y (horizontal()) then along x (vertical()). */
int orc_smooth(const float *in, int h, int w, float sigma, float *out) {
  if (h < 5 || w < 5) return -1;
  float c[17];
  smooth_coefficients(sigma, c);
  std::vector<float> tmp((size_t)h * w);
  for (int x = 0; x < w; ++x) iir_line(in + x, tmp.data() + x, h, w, c);
  for (int y = 0; y < h; ++y) iir_line(tmp.data() + (size_t)y * w, out + (size_t)y * w, w, 1, c);
  return 0;
}


void orc_patch_tables(float *mask, double *lcpos, double *lrpos) {
  /* initPatchMask(PATCH_SIZE), FeatureDescriptor.cpp:118-137 */
  const int center = kPatch >> 1;
  const float radius = center * center;
  const float sigma = 0.9 * radius;
  for (int i = 0; i < kPatch; ++i)
    for (int j = 0; j < kPatch; ++j) {
      const float disq = (i - center) * (i - center) + (j - center) * (j - center);
      mask[j * kPatch + i] = disq < radius ? std::exp(-disq / sigma) : 0.f;
    }
  /* precompute_patch_idx(.., iradius = PATCH_SIZE / 2, SrSize, ScSize), ShapeDescriptor.cpp:42-64 */
  const int ir = center;
  const float cspacing = kSc / (kM2Pi);
  for (int i = -ir; i <= ir; ++i)
    for (int j = -ir; j <= ir; ++j) {
      const int rpos = i, cpos = j;
      lcpos[(ir + j) * kPatch + (ir + i)] = (M_PI + std::atan2((double)rpos, (double)cpos)) * cspacing;
      lrpos[(ir + j) * kPatch + (ir + i)] =
          std::log(1 + std::sqrt((float)i * i + j * j) / ir) * kSr;
    }
}

/* KMAcomputeShape, ShapeDescriptor.cpp:168-261, on a normalised patch
 * [kPatch][kPatch]: gradients (dX2/dY2, gauss_iir.cpp:1182-1225), magnitude
 * and orientation, Canny edges (thresholds 5 and 15), log-polar histogram
 * of edge orientations weighted by the patch mask, L2 normalisation with a
 * 0.2 clip and integer quantisation (int)(512 v) capped at 255. */
void orc_shape_descriptor(const float *patch, float *vec) {
  float mask[kPatch * kPatch];
  double lc[kPatch * kPatch], lr[kPatch * kPatch];
  orc_patch_tables(mask, lc, lr);
  const int W = kPatch, H = kPatch;
  float dx[W * H], dy[W * H], grad[W * H], ori[W * H], edge[W * H];
  /* dX2 / dY2: central differences, zero on the border */
  for (int k = 0; k < W * H; ++k) dx[k] = dy[k] = 0;
  for (int y = 1; y < H - 1; ++y)
    for (int x = 1; x < W - 1; ++x) dx[y * W + x] = patch[y * W + x + 1] - patch[y * W + x - 1];
  for (int x = 1; x < W - 1; ++x)
    for (int y = 1; y < H - 1; ++y) dy[y * W + x] = patch[(y + 1) * W + x] - patch[(y - 1) * W + x];
  for (int k = 0; k < W * H; ++k) {
    grad[k] = std::sqrt(dx[k] * dx[k] + dy[k] * dy[k]);
    ori[k] = std::atan2(dy[k], dx[k]);
    edge[k] = 0;
  }
  canny(dx, dy, grad, edge, 5, 15);
  for (int k = 0; k < kShape; ++k) vec[k] = 0;
  const int ir = kPatch / 2;
  for (int i = -ir; i <= ir; ++i)
    for (int j = -ir; j <= ir; ++j) {
      const double lcpos = lc[(ir + j) * kPatch + (ir + i)];
      const double lrpos = lr[(ir + j) * kPatch + (ir + i)];
      const double rx = lrpos, cx = lcpos;
      if (!(rx > -1.0 && rx < (float)kSr && cx > -1.0 && cx < (float)kSc)) continue;
      /* KMAAddLogPolSample(vec, edge, ori, 0.0, ir + i, ir + j, ...), :126-164 */
      const int r = ir + i, c = ir + j;
      if (edge[r * W + c] < 1e-10) continue;
      const float mag = mask[r * W + c] * edge[r * W + c];
      float o = ori[r * W + c] - (float)0.0;
      while (o > M_PI) o -= M_PI;
      while (o < 0.0) o += M_PI;
      place(vec, mag, o, (float)lrpos, (float)lcpos);
    }
  normalize_vect(vec);
  bool changed = false;
  for (int i = 0; i < kShape; ++i)
    if (vec[i] > kMaxIndexVal) {
      vec[i] = kMaxIndexVal;
      changed = true;
    }
  if (changed) normalize_vect(vec);
  for (int i = 0; i < kShape; ++i) {
    const double s = 512.0 * vec[i];
    const int intval = std::isnan(s) ? INT_MIN : (int)s; /* x86-64 cvttsd2si */
    vec[i] = (255 < intval) ? 255 : intval;
  }
}

/* FeatureGrid(img_width, img_height, x_axis, y_axis, desc_step, desc_size)
 * (libPartDetect/FeatureGrid.cpp:22-97): the bounding box of the image in
 * the rotated frame and the grid size. */
void orc_feature_grid(int img_w, int img_h, const double *ax, const double *ay, double desc_step,
                      double *rect, int *nx, int *ny) {
  /* boost_math::inv for 2x2, boost_math.hpp:103-110, of T12 = [x_axis y_axis] */
  const double m00 = ax[0], m01 = ay[0], m10 = ax[1], m11 = ay[1];
  const double D = m00 * m11 - m10 * m01;
  const double t00 = m11 / D, t01 = -m01 / D, t10 = -m10 / D, t11 = m00 / D;
  const double cx[4] = {0, (double)img_w, (double)img_w, 0};
  const double cy[4] = {0, 0, (double)img_h, (double)img_h};
  double mnx = 0, mxx = 0, mny = 0, mxy = 0;
  for (int i = 0; i < 4; ++i) {
    const double px = t00 * cx[i] + t01 * cy[i], py = t10 * cx[i] + t11 * cy[i];
    if (i == 0) {
      mnx = mxx = px;
      mny = mxy = py;
      continue;
    }
    if (mnx > px) mnx = px;
    if (mxx < px) mxx = px;
    if (mny > py) mny = py;
    if (mxy < py) mxy = py;
  }
  rect[0] = mnx;
  rect[1] = mxx;
  rect[2] = mny;
  rect[3] = mxy;
  *nx = (int)std::floor(((mxx - mnx + 1) / desc_step)) + 1;
  *ny = (int)std::floor(((mxy - mny + 1) / desc_step)) + 1;
}

int orc_descriptor_grid_ex(const float *image, int img_h, int img_w, const double *ax,
                           const double *ay, double desc_step, int desc_size,
                           const float *detection_mask, const int *roi, float *cells,
                           uint8_t *valid) {
  double rect[4];
  int nx = 0, ny = 0;
  orc_feature_grid(img_w, img_h, ax, ay, desc_step, rect, &nx, &ny);
  const double patch_scale = (2 * desc_size + 1) / (float)kPatch;
  float mask[kPatch * kPatch];
  double lc[kPatch * kPatch], lr[kPatch * kPatch];
  orc_patch_tables(mask, lc, lr);
  /* smooth once for all descriptors if the patch is smaller than the window */
  std::vector<float> smoothed;
  if (patch_scale > 1.0) {
    smoothed.resize((size_t)img_h * img_w);
    if (orc_smooth(image, img_h, img_w, (float)patch_scale, smoothed.data())) return -2;
  }
  const Img src{img_w, img_h, patch_scale > 1.0 ? smoothed.data() : image};
  /* the ROI as QRect(x, y, width, height) holds it: right() = x + width - 1;
   * the default is QRect(0, 0, x() - 1, y() - 1) (partdetect_aux.cpp:44-55),
   * whose right() is x() - 2, so the reference tests it (:113-118) */
  const int rl = roi ? roi[0] : 0, rt = roi ? roi[1] : 0;
  const int rr = roi ? roi[0] + roi[2] - 1 : img_w - 2, rb = roi ? roi[1] + roi[3] - 1 : img_h - 2;
  const bool test_roi = !(rl == 0 && rr == img_w - 1 && rt == 0 && rb == img_h - 1);
  const unsigned uw = (unsigned)img_w, uh = (unsigned)img_h, ud = (unsigned)(desc_size + 1);
  float patch[kPatch * kPatch];
  for (int iy = 0; iy < ny; ++iy)
    for (int ix = 0; ix < nx; ++ix) {
      const size_t cell = (size_t)iy * nx + ix;
      valid[cell] = 0;
      std::memset(cells + cell * kShape, 0, kShape * sizeof(float));
      const double x2 = rect[0] + ix * desc_step, y2 = rect[2] + iy * desc_step;
      const double px = (0.0 + x2 * ax[0]) + y2 * ay[0];
      const double py = (0.0 + x2 * ax[1]) + y2 * ay[1];
      /* x() - (desc_size + 1) in the unsigned arithmetic of x() */
      if (!(px >= desc_size + 1 && px <= (double)(uw - ud) && py >= desc_size + 1 &&
            py <= (double)(uh - ud)))
        continue;
      /* detection_mask[imgpos(1)][imgpos(0)] == 0 skips the position (:132-138);
       * the double indices truncate */
      if (detection_mask && detection_mask[(size_t)(long)py * img_w + (size_t)(long)px] == 0)
        continue;
      if (test_roi && !(px >= rl && px <= rr && py >= rt && py <= rb)) continue;
      interpolate(src, (float)px, (float)py, (float)(patch_scale * ax[0]),
                  (float)(patch_scale * ay[0]), (float)(patch_scale * ax[1]),
                  (float)(patch_scale * ay[1]), patch);
      normalize_patch(patch, mask);
      orc_shape_descriptor(patch, cells + cell * kShape);
      valid[cell] = 1;
    }
  return 0;
}

int orc_descriptor_grid(const float *image, int img_h, int img_w, const double *ax,
                        const double *ay, double desc_step, int desc_size, float *cells,
                        uint8_t *valid) {
  return orc_descriptor_grid_ex(image, img_h, img_w, ax, ay, desc_step, desc_size, nullptr,
                                nullptr, cells, valid);
}

/* add_image_border2 (libKMA2/ImageContent/ImageContent.cpp:937-999): a
 * mirrored border of b pixels (b reduced to min(w, h) - 1 when too wide). */
int orc_add_border(const float *in, int h, int w, int b, float *out) {
  if (!(b < w && b < h)) b = std::min(w, h) - 1;
  const int W2 = w + 2 * b;
  for (int ix = 0; ix < w; ++ix)
    for (int iy = 0; iy < h; ++iy) out[(size_t)(b + iy) * W2 + b + ix] = in[(size_t)iy * w + ix];
  const int bx2 = b + w, by1 = b + 1, by2 = b + h;
  for (int bidx = 1; bidx <= b; ++bidx)
    for (int yidx = by1; yidx <= by2; ++yidx) {
      out[(size_t)(yidx - 1) * W2 + bidx - 1] = in[(size_t)(yidx - by1) * w + b - bidx];
      out[(size_t)(yidx - 1) * W2 + bx2 + bidx - 1] = in[(size_t)(yidx - by1) * w + w - bidx];
    }
  for (int bidx = 1; bidx <= b; ++bidx)
    for (int xidx = 0; xidx < W2; ++xidx) {
      out[(size_t)(bidx - 1) * W2 + xidx] = out[(size_t)(by1 + b - bidx - 1) * W2 + xidx];
      out[(size_t)(by2 + bidx - 1) * W2 + xidx] = out[(size_t)(by2 - bidx) * W2 + xidx];
    }
  return b;
}

}  // extern "C"

namespace {

/* hc::inverse (libBoostMath/homogeneous_coord.cpp:49-69) and the ublas 3 x 3
 * product, as in oracle.cpp. */
void hc_inv(const double *T, double *I) {
  double D = T[0] * T[4] - T[3] * T[1];
  I[0] = T[4] / D;
  I[1] = -T[1] / D;
  I[3] = -T[3] / D;
  I[4] = T[0] / D;
  double t0 = I[0] * T[2] + I[1] * T[5];
  double t1 = I[3] * T[2] + I[4] * T[5];
  I[2] = -t0;
  I[5] = -t1;
  I[6] = 0;
  I[7] = 0;
  I[8] = 1;
}
int partdetect_scale(const orc_exp *e, int si, const orc_models *m, const int *window_size,
                     const double *pos_offset, int desc_step0, int desc_size0, double ratio,
                     const float *image, int h, int w, int flip, const float *mask,
                     float *log_unary);

void mul3(const double *A, const double *B, double *Cm) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = 0;
      for (int k = 0; k < 3; ++k) t += A[3 * i + k] * B[3 * k + j];
      Cm[3 * i + j] = t;
    }
}

}  // namespace

extern "C" {

/* partdetect_dense for one image, one scale, in-memory path
 * (libPartDetect/partdetect_test.cpp:53-294) followed by clip_scores_fill +
 * computeLogGrid (objectdetect_findrot.cpp:834-845): see oracle.h. */
int orc_partdetect_masked(const orc_exp *e, const orc_models *m, const int *window_size,
                          const double *pos_offset, int desc_step0, int desc_size0, double ratio,
                          const float *image, int h, int w, int flip,
                          const float *detection_mask, float *log_unary) {
  const int S = n_scales_desc(e);
  if (S > 1 && e->min_object_scale == e->max_object_scale) return -1;
  for (int si = 0; si < S; ++si) {
    const int rc = partdetect_scale(e, si, m, window_size, pos_offset, desc_step0, desc_size0,
                                    ratio, image, h, w, flip,
                                    detection_mask ? detection_mask + (size_t)si * h * w : nullptr,
                                    log_unary);
    if (rc) return rc;
  }
  return 0;
}

int orc_partdetect(const orc_exp *e, const orc_models *m, const int *window_size,
                   const double *pos_offset, int desc_step0, int desc_size0, double ratio,
                   const float *image, int h, int w, int flip, float *log_unary) {
  return orc_partdetect_masked(e, m, window_size, pos_offset, desc_step0, desc_size0, ratio,
                               image, h, w, flip, nullptr, log_unary);
}

}  // extern "C"

namespace {

/* one scale of partdetect_dense: log unaries of scale si into
 * log_unary [n][S][R][h][w] */
int partdetect_scale(const orc_exp *e, int si, const orc_models *m, const int *window_size,
                     const double *pos_offset, int desc_step0, int desc_size0, double ratio,
                     const float *image, int h, int w, int flip, const float *mask,
                     float *log_unary) {
  const int S = n_scales_desc(e);
  const double scale = scale_value(e, si);
  const int R = e->num_rotation_steps, n = m->n_parts;
  const double desc_step = scale * desc_step0;
  const int desc_size = (int)std::floor(scale * desc_size0 + 0.5); /* boost_math::round */
  double max_part_diag = 0;
  for (int c = 0; c < n; ++c) {
    const int wx = window_size[2 * c], wy = window_size[2 * c + 1];
    const double d = std::sqrt((double)(wx * wx + wy * wy));
    if (d > max_part_diag) max_part_diag = d;
  }
  int border = (int)std::ceil(desc_size + 0.5 * scale * max_part_diag);
  const int b = (border < w && border < h) ? border : std::min(w, h) - 1;
  const int eh = h + 2 * b, ew = w + 2 * b;
  std::vector<float> ext((size_t)eh * ew);
  orc_add_border(image, h, w, b, ext.data());
  /* this scale's detection mask placed in a zero array of the bordered
   * image's size (partdetect_test.cpp:135-146) */
  std::vector<float> ext_mask;
  if (mask) {
    ext_mask.assign((size_t)eh * ew, 0.f);
    for (int y = 0; y < h; ++y)
      std::memcpy(ext_mask.data() + (size_t)(y + b) * ew + b, mask + (size_t)y * w,
                  (size_t)w * sizeof(float));
  }
  double window_step = ratio * desc_step;
  if (window_step < 1) window_step = 1;
  const double grid_step = desc_step / window_step;
  const size_t HW = (size_t)h * w;
  for (int r = 0; r < R; ++r) {
    double rotation = rot_value(e, r);
    rotation *= M_PI / 180.0;
    double ax[2] = {std::cos(rotation), std::sin(rotation)};
    const double ay[2] = {-std::sin(rotation), std::cos(rotation)};
    if (flip) {
      ax[0] = -ax[0];
      ax[1] = -ax[1];
    }
    double rect[4];
    int nx = 0, ny = 0;
    orc_feature_grid(ew, eh, ax, ay, window_step, rect, &nx, &ny);
    std::vector<float> cells((size_t)nx * ny * kShape);
    std::vector<uint8_t> valid((size_t)nx * ny);
    if (orc_descriptor_grid_ex(ext.data(), eh, ew, ax, ay, window_step, desc_size,
                               mask ? ext_mask.data() : nullptr, nullptr, cells.data(),
                               valid.data()))
      return -2;
    const double T32[9] = {1, 0, -rect[0], 0, 1, -rect[2], 0, 0, 1};
    double T23[9];
    hc_inv(T32, T23);
    const double Ti2[9] = {ax[0], ay[0], 0, ax[1], ay[1], 0, 0, 0, 1};
    const double Tie[9] = {1, 0, (double)-b, 0, 1, (double)-b, 0, 0, 1};
    double Ti2e[9];
    mul3(Tie, Ti2, Ti2e);
    for (int c = 0; c < n; ++c) {
      const int gx = window_size[2 * c] / desc_step0 + 1, gy = window_size[2 * c + 1] / desc_step0 + 1;
      const size_t so = (size_t)c * m->n_stumps;
      std::vector<float> grid((size_t)nx * ny);
      orc_score_grid_window(m->f + so, m->p + so, m->theta + so, m->alpha + so, m->n_stumps,
                            m->sum_alpha[c], cells.data(), valid.data(), ny, nx, kShape, gx, gy,
                            grid_step, 1, grid.data());
      /* computeScoreGrid's transforms, :379-403 */
      double T3g[9] = {window_step, 0, 0, 0, window_step, 0, 0, 0, 1};
      T3g[2] = scale * pos_offset[2 * c];
      T3g[5] = scale * pos_offset[2 * c + 1];
      double T2g[9];
      mul3(T23, T3g, T2g);
      /* squeezeScoreGrid, :407-449 */
      int bb[4];
      std::vector<float> sq = grid;
      int sny = ny, snx = nx;
      if (orc_squeeze_bbox(grid.data(), ny, nx, bb)) {
        snx = bb[2] - bb[0] + 1;
        sny = bb[3] - bb[1] + 1;
        sq.assign((size_t)snx * sny, 0.f);
        for (int y = 0; y < sny; ++y)
          for (int x = 0; x < snx; ++x)
            sq[(size_t)y * snx + x] = grid[(size_t)(y + bb[1]) * nx + x + bb[0]];
        const double Tg4[9] = {1, 0, (double)bb[0], 0, 1, (double)bb[1], 0, 0, 1};
        double M[9];
        mul3(T2g, Tg4, M);
        std::memcpy(T2g, M, sizeof M);
      }
      double Tig[9];
      mul3(Ti2e, T2g, Tig);
      float *out = log_unary + (((size_t)c * S + si) * R + r) * HW;
      orc_transform_grid(sq.data(), sny, snx, out, h, w, Tig, 0.f, 2);
      orc_clip_log(out, (int64_t)HW);
    }
  }
  return 0;
}

}  // namespace
