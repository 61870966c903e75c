/*
 * oracle.cpp -- CPU restatement of partapp's inference hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Compiled with -ffp-contract=off
 * so that every a*b+c is the two rounded operations the 2013 x86 build of the
 * reference performed (no fused multiply-add), on x86 and on Arm alike.
 *
 * Numeric conventions of the FP32 flavour (the reference stores every map as
 * boost::multi_array<float,...>):
 *   - exp/log of a float element are evaluated in double and rounded to
 *     float (the unqualified exp()/log() in libMultiArray/multi_array_op.hpp
 *     resolve to the double C functions);
 *   - cblas_sdot is restated as a sequential float dot product; its
 *     summation order is implementation-defined in BLAS, so sums are only
 *     compared within a tolerance.
 * The FP64 flavour runs the identical algorithm on doubles.
 */
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <utility>
#include <vector>

namespace {

/* libBoostMath/boost_math.h:23 */
const double LOG_ZERO = -1e6;
/* libPartDetect/partdetect.h:45 */
const float NO_CLASS_VALUE = 0.0f;

/* boost_math::round, libBoostMath/boost_math.hpp:35-37 */
inline int bm_round(double v) { return (int)std::floor(v + 0.5); }

/* value_from_index, libPartApp/partapp_aux.hpp:45-58 */
double value_from_index(double minval, double maxval, double num_steps, int idx) {
  if (minval == maxval) return minval;
  double step_size = (maxval - minval) / num_steps;
  return minval + step_size * (0.5 + idx);
}

/* index_from_value, libPartApp/partapp_aux.hpp:23-43 */
int index_from_value(double minval, double maxval, double num_steps, double val) {
  if (minval == maxval) return 0;
  double step_size = (maxval - minval) / num_steps;
  return (int)std::floor((val - minval) / step_size);
}

/* rot_from_index / index_from_rot, libPartApp/partapp_aux.hpp:93-129 */
double rot_from_index(const orc_exp *e, int idx) {
  return value_from_index(e->min_part_rotation, e->max_part_rotation,
                          (double)(unsigned)e->num_rotation_steps, idx);
}
int index_from_rot(const orc_exp *e, double rot) {
  return index_from_value(e->min_part_rotation, e->max_part_rotation,
                          (double)(unsigned)e->num_rotation_steps, rot);
}
/* ExpParam::num_scale_steps (ExpParam.proto:191, default 1); 0 reads as 1 */
int n_scales(const orc_exp *e) { return e->num_scale_steps > 1 ? e->num_scale_steps : 1; }

/* scale_from_index, partapp_aux.hpp:86-92 */
double scale_from_index(const orc_exp *e, int idx) {
  return value_from_index(e->min_object_scale, e->max_object_scale,
                          (double)n_scales(e), idx);
}

template <class T> struct Num;
template <> struct Num<float> {
  static float ex(float x) { return (float)std::exp((double)x); }
  static float lg(float x) { return (float)std::log((double)x); }
};
template <> struct Num<double> {
  static double ex(double x) { return std::exp(x); }
  static double lg(double x) { return std::log(x); }
};

/* get_gaussian_filter, libBoostMath/boost_math.cpp:104-117 (bNormalize =
 * false on this path, objectdetect_findrot.cpp:370-371). */
std::vector<double> gaussian_filter(double sigma) {
  int ksize = (int)std::floor(3 * sigma + 0.5);
  std::vector<double> f(2 * ksize + 1);
  f[ksize] = 1.0;
  for (int i = 1; i <= ksize; ++i) {
    f[ksize + i] = std::exp(-i * i / (2 * sigma * sigma));
    f[ksize - i] = f[ksize + i];
  }
  return f;
}

/* Sequential dot product standing in for cblas_sdot. */
template <class T>
inline T dot(int n, const T *x, int incx, const T *y) {
  T s = 0;
  for (int i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[i];
  return s;
}

/* The offset a joint applies at rotation index r: the vector
 * prod(prod(R(alpha), S(scale)), (ox, oy, 0)) of
 * objectdetect_findrot.cpp:348-351 / 439-441, evaluated in the same
 * operation order (hc::get_rotation_matrix, homogeneous_coord.cpp:81-93). */
void rotate_offset(const orc_exp *e, int r, double scale, const double *o,
                   double &dx, double &dy) {
  float alpha = (float)(rot_from_index(e, r) * M_PI / 180.0);
  double ca = std::cos((double)alpha), sa = std::sin((double)alpha);
  double t00 = ca * scale, t01 = (-sa) * scale;
  double t10 = sa * scale, t11 = ca * scale;
  dx = t00 * o[0] + t01 * o[1];
  dy = t10 * o[0] + t11 * o[1];
}

/* transform_grid_fixed_size(..., translation(tx, ty), default, TM_NEAREST)
 * (multi_array_transform.hpp:194-215): with T13 = inverse(T21) the source of
 * output cell (x3, y3) is floor((x3 + (-tx)) + 0.5). */
template <class T>
void shift_nearest(const T *src, T *dst, int H, int W, double tx, double ty,
                   T def) {
  const double ax = -tx, ay = -ty;
  for (int x3 = 0; x3 < W; ++x3)
    for (int y3 = 0; y3 < H; ++y3) {
      T v = def;
      double x1 = (double)x3 + ax;
      double y1 = (double)y3 + ay;
      int ix1 = (int)std::floor(x1 + 0.5);
      int iy1 = (int)std::floor(y1 + 0.5);
      if (ix1 >= 0 && ix1 < W && iy1 >= 0 && iy1 < H) v = src[(size_t)iy1 * W + ix1];
      dst[(size_t)y3 * W + x3] = v;
    }
}

/* computeLogGrid, multi_array_op.hpp:154-167 */
template <class T> void log_grid(T *d, size_t n) {
  for (size_t i = 0; i < n; ++i) d[i] = (d[i] == 0) ? (T)LOG_ZERO : Num<T>::lg(d[i]);
}

/* hc::inverse, libBoostMath/homogeneous_coord.cpp:49-69 */
void hc_inverse3(const double *T, double *I) {
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

/* ublas prod of two 3x3 matrices (row-major): C(i,j) = sum_k A(i,k) B(k,j),
 * accumulated k = 0, 1, 2. */
void prod3(const double *A, const double *B, double *Cm) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = 0;
      for (int k = 0; k < 3; ++k) t += A[3 * i + k] * B[3 * k + j];
      Cm[3 * i + j] = t;
    }
}

/* boost_math::eig2d, libBoostMath/boost_math.cpp:40-99: E = (smallest,
 * largest) eigenvalue, V columns = eigenvectors, V(0,0) = v11. */
void eig2d(const double *M, double *V, double *E) {
  double m11 = M[0], m12 = M[1], m22 = M[3];
  double e1, e2, v11, v21;
  if (m12 != 0) {
    double sqrtD = std::sqrt((m11 - m22) * (m11 - m22) + 4 * m12 * m12);
    e1 = 0.5 * (m11 + m22 - sqrtD);
    e2 = 0.5 * (m11 + m22 + sqrtD);
    v11 = 0.5 * (m11 - m22 - sqrtD) / m12;
    v21 = 1;
  } else if (m11 < m22) {
    e1 = m11; e2 = m22; v11 = 1; v21 = 0;
  } else {
    e1 = m22; e2 = m11; v11 = 0; v21 = 1;
  }
  double norm_v1 = std::sqrt(v11 * v11 + v21 * v21);
  v11 /= norm_v1;
  v21 /= norm_v1;
  V[0] = v11;   /* V(0,0) */
  V[1] = -v21;  /* V(0,1) = v12 */
  V[2] = v21;   /* V(1,0) */
  V[3] = v11;   /* V(1,1) = v22 */
  E[0] = e1;
  E[1] = e2;
}

/* hc::get_transformed_bbox, homogeneous_coord.cpp:140-156 */
void transformed_bbox(const double *T21, int in_w, int in_h, double &minx, double &miny,
                      double &maxx, double &maxy) {
  const double px[4] = {0, (double)(in_w - 1), 0, (double)(in_w - 1)};
  const double py[4] = {0, 0, (double)(in_h - 1), (double)(in_h - 1)};
  double xs[4], ys[4];
  for (int c = 0; c < 4; ++c) {
    xs[c] = T21[0] * px[c] + T21[1] * py[c] + T21[2] * 1.0;
    ys[c] = T21[3] * px[c] + T21[4] * py[c] + T21[5] * 1.0;
  }
  minx = *std::min_element(xs, xs + 4);
  maxx = *std::max_element(xs, xs + 4);
  miny = *std::min_element(ys, ys + 4);
  maxy = *std::max_element(ys, ys + 4);
}

/* The bilinear branch of transform_grid_helper
 * (multi_array_transform.hpp:194-238) with the output -> input map T13
 * given: exact-hit shortcut, last row/column left at the default. */
template <class T>
void bilinear_map(const T *gin, int in_h, int in_w, T *gout, int out_h, int out_w,
                  const double *T13, T def) {
  const T eps10 = 10 * std::numeric_limits<T>::epsilon();
  for (int x3 = 0; x3 < out_w; ++x3)
    for (int y3 = 0; y3 < out_h; ++y3) {
      T o = def;
      double x1 = T13[0] * x3 + T13[1] * y3 + T13[2];
      double y1 = T13[3] * x3 + T13[4] * y3 + T13[5];
      int ix1 = (int)std::floor(x1), iy1 = (int)std::floor(y1);
      if (ix1 >= 0 && ix1 < in_w && iy1 >= 0 && iy1 < in_h) {
        T a = (T)(x1 - ix1), b = (T)(y1 - iy1);
        if (a < eps10 && b < eps10) {
          o = gin[(size_t)iy1 * in_w + ix1];
        } else if (ix1 < in_w - 1 && iy1 < in_h - 1) {
          const T *g0 = gin + (size_t)iy1 * in_w + ix1, *g1 = g0 + in_w;
          const T one = 1;
          o = (one - b) * (one - a) * g0[0] + (one - b) * a * g0[1] + b * (one - a) * g1[0] +
              b * a * g1[1];
        }
      }
      gout[(size_t)y3 * out_w + x3] = o;
    }
}

/* gaussFilterDiag2d, multi_array_filter.hpp:212-321: x pass then y pass,
 * taps truncated at the border, sequential float dots. */
template <class T>
void gauss_diag(const T *in, T *out, int H, int W, double sigma_x, double sigma_y) {
  std::vector<double> fxd = gaussian_filter(sigma_x), fyd = gaussian_filter(sigma_y);
  std::vector<T> fx(fxd.begin(), fxd.end()), fy(fyd.begin(), fyd.end());
  const int kx = ((int)fx.size() - 1) / 2, ky = ((int)fy.size() - 1) / 2;
  std::vector<T> sm((size_t)H * W);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      int n1 = std::max(0, x - kx), n2 = std::min(W - 1, x + kx);
      sm[(size_t)y * W + x] = dot(n2 - n1 + 1, in + (size_t)y * W + n1, 1, fx.data() + (n1 - (x - kx)));
    }
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      int n1 = std::max(0, y - ky), n2 = std::min(H - 1, y + ky);
      out[(size_t)y * W + x] = dot(n2 - n1 + 1, sm.data() + (size_t)n1 * W + x, W, fy.data() + (n1 - (y - ky)));
    }
}

/* The TM_DIRECT branch of transform_grid_helper (multi_array_transform.hpp:
 * 173-193) with the input -> output map T31: every input cell that is not the
 * default lands on its nearest output cell, later cells (x outer, y inner)
 * overwriting earlier ones; unreached cells keep the default. */
template <class T>
void direct_map(const T *gin, int in_h, int in_w, T *gout, int out_h, int out_w,
                const double *T31, T def) {
  std::fill(gout, gout + (size_t)out_h * out_w, def);
  for (int x1 = 0; x1 < in_w; ++x1)
    for (int y1 = 0; y1 < in_h; ++y1) {
      const T v = gin[(size_t)y1 * in_w + x1];
      if (v != def) {
        double x3 = T31[0] * x1 + T31[1] * y1 + T31[2];
        double y3 = T31[3] * x1 + T31[4] * y1 + T31[5];
        int ix3 = (int)std::floor(x3 + 0.5), iy3 = (int)std::floor(y3 + 0.5);
        if (ix3 >= 0 && ix3 < out_w && iy3 >= 0 && iy3 < out_h) gout[(size_t)iy3 * out_w + ix3] = v;
      }
    }
}

/* gaussFilter2dOffset with a zero offset, multi_array_filter.hpp:335-369:
 * bilinear forward rotation, or TM_DIRECT when bIsSparse. */
template <class T>
void gauss_full(const T *in, T *out, int H, int W, const double *Cs, bool sparse) {
  double V[4], E[2];
  eig2d(Cs, V, E);
  const double T21[9] = {V[0], V[2], 0, V[1], V[3], 0, 0, 0, 1};  /* [trans(V) | 0] */
  double minx, miny, maxx, maxy;
  transformed_bbox(T21, W, H, minx, miny, maxx, maxy);
  const int ow = (int)std::ceil(maxx - minx), oh = (int)std::ceil(maxy - miny);
  const double T23[9] = {1, 0, minx, 0, 1, miny, 0, 0, 1};
  double T12[9], T13[9];
  hc_inverse3(T21, T12);
  prod3(T12, T23, T13);
  std::vector<T> g((size_t)oh * ow), gs((size_t)oh * ow);
  if (sparse) {
    const double T32[9] = {1, 0, -minx, 0, 1, -miny, 0, 0, 1};
    double T31[9];
    prod3(T32, T21, T31);
    direct_map(in, H, W, g.data(), oh, ow, T31, (T)0);
  } else {
    bilinear_map(in, H, W, g.data(), oh, ow, T13, (T)0);
  }
  gauss_diag(g.data(), gs.data(), oh, ow, std::sqrt(E[0]), std::sqrt(E[1]));
  const double mz = -0.0;
  const double T42[9] = {V[0], V[1], mz, V[2], V[3], mz, 0, 0, 1};
  double T43[9], Tb[9], Tbb[9];
  prod3(T42, T23, T43);
  hc_inverse3(T43, Tb);
  const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  prod3(Tb, I3, Tbb);
  bilinear_map(gs.data(), oh, ow, out, H, W, Tbb, (T)0);
}

/* computeRotJointMarginal, objectdetect_findrot.cpp:292-456. */
template <class T>
int rot_joint_marginal(const orc_exp *e, const T *child, T *parent, int R, int H,
                       int W, const double *oc, const double *op,
                       const double *C, double rot_mean, double rot_sigma,
                       double scale, bool sparse) {
  const size_t HW = (size_t)H * W, N = HW * R;
  if (R < 2 || H < 1 || W < 1) return -1;
  const bool diag = (C[1] == 0 && C[2] == 0);
  if (!diag && C[1] != C[2]) return -1; /* eig2d asserts symmetry */
  if (diag && !(C[0] > 0 && C[3] > 0)) return -1;

  /* getMinMax, multi_array_op.hpp:61-77 */
  T in_M = -std::numeric_limits<T>::infinity();
  for (size_t i = 0; i < N; ++i)
    if (child[i] > in_M) in_M = child[i];

  /* :319-326 */
  float step_f = (e->max_part_rotation - e->min_part_rotation) /
                 (float)(unsigned)e->num_rotation_steps;
  double rot_step_size = step_f;
  rot_step_size *= M_PI / 180.0;
  double rot_sigma_idx = rot_sigma / rot_step_size;
  int rot_mean_idx = bm_round(-rot_mean / rot_step_size);

  std::vector<T> j10(N, (T)LOG_ZERO), j01(N, (T)LOG_ZERO);

  /* :345-359 */
  for (int r = 0; r < R; ++r) {
    int r_out = r + rot_mean_idx;
    if (r_out >= 0 && r_out < R) {
      double dx, dy;
      rotate_offset(e, r, scale, oc, dx, dy);
      shift_nearest(child + r * HW, j10.data() + r_out * HW, H, W, dx, dy, (T)LOG_ZERO);
    }
  }

  /* addGrid1(-in_M) + computeExpGrid, :362-365 */
  const T neg_M = -in_M;
  for (size_t i = 0; i < N; ++i) j10[i] = Num<T>::ex(j10[i] + neg_M);

  /* rotation dimension, :373-420 */
  std::vector<T> rot_res(N, (T)0);
  if (rot_sigma > 0) {
    std::vector<double> f_rot = gaussian_filter(rot_sigma_idx);
    int firstidx = 0;
    int f_rot_size = (int)f_rot.size();
    if (f_rot_size >= R) {
      int crot = f_rot_size / 2;
      f_rot_size = (R % 2 == 1) ? R - 2 : R - 1;
      firstidx = crot - f_rot_size / 2;
    }
    std::vector<T> ff(f_rot_size);
    for (int idx = firstidx; idx < firstidx + f_rot_size; ++idx) ff[idx - firstidx] = (T)f_rot[idx];
    /* grid_filter_1d_blas_wraparound, multi_array_filter.hpp:116-155 */
    const int nx = (f_rot_size - 1) / 2;
    std::vector<T> g(R + 2 * nx);
    for (int x = 0; x < W; ++x)
      for (int y = 0; y < H; ++y) {
        const size_t off = (size_t)y * W + x;
        for (int r = 0; r < R; ++r) g[nx + r] = j10[r * HW + off];
        for (int idx = 0; idx < nx; ++idx) g[nx - 1 - idx] = j10[(R - 1 - idx) * HW + off];
        for (int idx = 0; idx < nx; ++idx) g[nx + R + idx] = j10[idx * HW + off];
        for (int r = 0; r < R; ++r) rot_res[r * HW + off] = dot(f_rot_size, &g[r], 1, ff.data());
      }
  } else if (rot_sigma == 0) {
    rot_res = j10;
  }

  /* x/y dimensions: gaussFilter2d -> gaussFilterDiag2d, :423-429 and
   * multi_array_filter.hpp:212-321, 375-388 */
  const double sc2 = scale * scale;
  const double Cs[4] = {sc2 * C[0], sc2 * C[1], sc2 * C[2], sc2 * C[3]};  /* square(scale)*C */
  for (int r = 0; r < R; ++r) {
    const T *in = rot_res.data() + r * HW;
    T *out = j01.data() + r * HW;
    if (diag)
      gauss_diag(in, out, H, W, std::sqrt(Cs[0]), std::sqrt(Cs[3]));
    else
      gauss_full(in, out, H, W, Cs, sparse);
  }

  /* computeLogGrid + addGrid1(in_M), :432-435 */
  log_grid(j01.data(), N);
  for (size_t i = 0; i < N; ++i) j01[i] = j01[i] + in_M;

  /* :438-448 */
  for (int r = 0; r < R; ++r) {
    double dx, dy;
    rotate_offset(e, r, scale, op, dx, dy);
    shift_nearest(j01.data() + r * HW, parent + r * HW, H, W, -dx, -dy, (T)LOG_ZERO);
  }
  return 0;
}

/* findLocalMax, objectdetect_aux.cpp:193-264 */
template <class T>
std::vector<std::array<double, 4>> find_local_max(const T *g, int S, int H, int W, int max_n) {
  std::vector<std::array<double, 4>> lm;
  const size_t HW = (size_t)H * W;
  auto at = [&](int s, int y, int x) { return g[s * HW + (size_t)y * W + x]; };
  for (int s = 0; s < S; ++s)
    for (int x = 0; x < W; ++x)
      for (int y = 0; y < H; ++y) {
        bool ok = true;
        const T v = at(s, y, x);
        for (int dy = -1; dy <= 1 && ok; ++dy)
          for (int dx = -1; dx <= 1 && ok; ++dx) {
            int xp = x + dx, yp = y + dy;
            if (xp >= 0 && xp < W && yp >= 0 && yp < H && !(dx == 0 && dy == 0))
              if (at(s, yp, xp) > v) ok = false;
          }
        if (ok && s > 0) ok = at(s - 1, y, x) < v;
        if (ok && s < S - 1) ok = at(s + 1, y, x) < v;
        if (ok) lm.push_back({(double)s, (double)x, (double)y, (double)v});
      }
  if ((int)lm.size() > max_n) {
    std::vector<std::pair<float, int>> validx;
    validx.reserve(lm.size());
    for (int i = 0; i < (int)lm.size(); ++i) validx.emplace_back((float)lm[i][3], i);
    std::stable_sort(validx.begin(), validx.end(),
                     [](const std::pair<float, int> &a, const std::pair<float, int> &b) {
                       return a.first > b.first;
                     });
    std::vector<std::array<double, 4>> top;
    top.reserve(max_n);
    for (int i = 0; i < max_n; ++i) top.push_back(lm[validx[i].second]);
    lm.swap(top);
  }
  return lm;
}

/* get_incoming_joints, objectdetect_findrot.cpp:59-71 */
void incoming(const orc_tree *t, int cur, std::vector<int> &ch, std::vector<int> &js) {
  ch.clear();
  js.clear();
  for (int j = 0; j < t->n_joints; ++j)
    if (t->parent[j] == cur) {
      ch.push_back(t->child[j]);
      js.push_back(j);
    }
}

template <class T> void add_grid(std::vector<T> &a, const std::vector<T> &b) {
  for (size_t i = 0; i < a.size(); ++i) a[i] += b[i];
}

/* PartHyp(exp_param, scaleidx, rotidx, x, y, score).toVect(),
 * objectdetect.h:95-159 */
void part_hyp_vect(const orc_exp *e, int rotidx, int x, int y, float score, float *o,
                   int scaleidx = 0) {
  o[0] = (float)scaleidx;
  o[1] = (float)scale_from_index(e, scaleidx);
  o[2] = (float)rotidx;
  o[3] = (float)rot_from_index(e, rotidx);
  o[4] = (float)x;
  o[5] = (float)y;
  o[6] = score;
}

/* first strict maximum over the flat [R][H][W] index,
 * objectdetect_findrot.cpp:261-277 */
template <class T>
void best_hyp(const orc_exp *e, const T *g, int R, int H, int W, float *o, int scaleidx) {
  float bestval = (float)-std::numeric_limits<double>::max(); /* -DBL_MAX */
  T bestv = (T)bestval;
  long bestidx = -1;
  const long N = (long)R * H * W;
  for (long i = 0; i < N; ++i)
    if (g[i] > bestv) {
      bestv = g[i];
      bestidx = i;
    }
  if (bestidx < 0) bestidx = 0;
  int r = (int)(bestidx / ((long)H * W));
  long rem = bestidx % ((long)H * W);
  int x = (int)(rem % W), y = (int)(rem / W);
  part_hyp_vect(e, r, x, y, (float)bestv, o, scaleidx);
}

/* One scale of computeRootPosteriorRot: the upward pass (:578-658) and
 * computePartMarginals (:124-236) at `scale`; post[p] receives the final
 * log marginals. */
template <class T>
int ps_one_scale(const orc_exp *e, const orc_tree *t, const std::vector<std::vector<T>> &unary,
                 int H, int W, double scale, std::vector<std::vector<T>> &post) {
  const int P = t->n_parts, R = e->num_rotation_steps;
  const size_t N = (size_t)H * W * R;
  const int root = t->root;
  post.assign(P, std::vector<T>(N, (T)0));
  std::vector<std::vector<T>> from_root(P, std::vector<T>(N, (T)0));
  std::vector<T> msg(N);
  std::vector<int> ch, js;

  /* upward pass, :578-658 */
  std::vector<bool> done(P, false);
  std::vector<int> stack{root};
  while (!stack.empty()) {
    int cur = stack.back();
    stack.pop_back();
    bool can = true;
    for (int j = 0; j < t->n_joints; ++j)
      if (t->parent[j] == cur && !done[t->child[j]]) {
        can = false;
        stack.push_back(cur);
        stack.push_back(t->child[j]);
        break;
      }
    if (!can) continue;
    incoming(t, cur, ch, js);
    for (size_t i = 0; i < ch.size(); ++i) {
      int c = ch[i], j = js[i];
      int rc = rot_joint_marginal<T>(e, post[c].data(), msg.data(), R, H, W, t->offset_c + 2 * j,
                                     t->offset_p + 2 * j, t->C + 4 * j, t->rot_mean[j],
                                     t->rot_sigma[j], scale, e->sparse_up != 0);
      if (rc) return rc;
      add_grid(post[cur], msg);
      if (cur == root)
        for (size_t i2 = 0; i2 < ch.size(); ++i2)
          if (i2 != i) add_grid(from_root[ch[i2]], msg);
    }
    add_grid(post[cur], unary[cur]);
    done[cur] = true;
  }

  /* computePartMarginals, :124-236 */
  incoming(t, root, ch, js);
  std::vector<int> stack2;
  std::vector<int> rch = ch, rjs = js;
  for (size_t i = 0; i < rch.size(); ++i) {
    int c = rch[i], j = rjs[i];
    add_grid(from_root[c], unary[root]);
    int rc = rot_joint_marginal<T>(e, from_root[c].data(), msg.data(), R, H, W, t->offset_p + 2 * j,
                                   t->offset_c + 2 * j, t->C + 4 * j, -t->rot_mean[j],
                                   t->rot_sigma[j], scale, false);
    if (rc) return rc;
    from_root[c] = msg;
    stack2.push_back(c);
  }
  while (!stack2.empty()) {
    int cur = stack2.back();
    stack2.pop_back();
    add_grid(post[cur], from_root[cur]);
    incoming(t, cur, ch, js);
    if (ch.size() > 1) return -3; /* assert(all_children.size() <= 1), :210 */
    if (ch.size() == 1) {
      int c = ch[0], j = js[0];
      std::vector<T> tmp = unary[cur];
      add_grid(tmp, from_root[cur]);
      int rc = rot_joint_marginal<T>(e, tmp.data(), from_root[c].data(), R, H, W,
                                     t->offset_p + 2 * j, t->offset_c + 2 * j, t->C + 4 * j,
                                     -t->rot_mean[j], t->rot_sigma[j], scale, false);
      if (rc) return rc;
      stack2.push_back(c);
    }
  }
  return 0;
}

/* computeRootPosteriorRot (objectdetect_findrot.cpp:470-727) over all
 * num_scale_steps scales, each an independent pass at its own scale (the
 * loop :503-678).  log_unary [P][S][R][H][W]; log_marg [P][S][R][H][W];
 * root_post [S][H][W].  best_conf and part_hyps are those of the last scale
 * (computePartMarginals clears best_part_hyp on every scale, :254-258); the
 * root hypotheses are the local maxima of the [S][H][W] root posterior with
 * scale neighbours (:1037-1038).  Without pairwise terms the reference
 * reads scale 0 only (getMaxStates, :73-110). */
template <class T>
int ps_infer(const orc_exp *e, const orc_tree *t, const T *log_unary, int H, int W,
             T *log_marg, float *best_conf, T *root_post_out, float *part_hyps,
             int *n_part_hyps, float *root_hyps, int *n_root_hyps) {
  const int P = t->n_parts, R = e->num_rotation_steps, S = n_scales(e);
  const size_t HW = (size_t)H * W, N = HW * R;
  const int root = t->root;
  if (P < 1 || root < 0 || root >= P || t->n_joints != P - 1) return -1;
  if (S > 1 && e->min_object_scale == e->max_object_scale) return -1; /* :33-38 asserts */

  /* unary[s][p] */
  std::vector<std::vector<std::vector<T>>> unary(S, std::vector<std::vector<T>>(P));
  for (int sc = 0; sc < S; ++sc)
    for (int p = 0; p < P; ++p)
      unary[sc][p].assign(log_unary + ((size_t)p * S + sc) * N,
                          log_unary + ((size_t)p * S + sc + 1) * N);

  for (int sc = 0; sc < S; ++sc) {
    /* enforce upright orientation, objectdetect_findrot.cpp:509-523 */
    for (int p = 0; p < P; ++p)
      if (t->is_upright[p])
        for (int r = 0; r < R; ++r) {
          double cur_rot = rot_from_index(e, r);
          if (!(std::fabs(cur_rot) < 15.0))
            std::fill(unary[sc][p].begin() + r * HW, unary[sc][p].begin() + (r + 1) * HW,
                      (T)LOG_ZERO);
        }
    /* strip border detections of the root, :528-551 */
    if (e->strip_border_detections > 0) {
      int sw = (int)(e->strip_border_detections * W);
      for (int r = 0; r < R; ++r)
        for (int y = 0; y < H; ++y) {
          T *row = unary[sc][root].data() + r * HW + (size_t)y * W;
          for (int x = 0; x < sw; ++x) row[x] = (T)LOG_ZERO;
          for (int x = W - sw; x < W; ++x) row[x] = (T)LOG_ZERO;
        }
    }
  }

  const int hyp_scale = e->use_pairwise ? S - 1 : 0;
  std::vector<T> root_full(e->use_pairwise ? (size_t)S * HW : 0);
  std::vector<std::vector<T>> post;
  for (int sc = 0; sc < S; ++sc) {
    if (e->use_pairwise) {
      int rc = ps_one_scale<T>(e, t, unary[sc], H, W, scale_from_index(e, sc), post);
      if (rc) return rc;
    } else {
      post = unary[sc]; /* getMaxStates: the marginals are the unaries */
    }
    for (int p = 0; p < P; ++p) {
      if (log_marg) std::copy(post[p].begin(), post[p].end(), log_marg + ((size_t)p * S + sc) * N);
      if (sc != hyp_scale) continue;
      if (best_conf) best_hyp(e, post[p].data(), R, H, W, best_conf + 7 * p, sc);
      if (part_hyps || n_part_hyps) {
        const int K = e->max_local_max;
        auto lm = find_local_max(post[p].data(), R, H, W, K);
        if (n_part_hyps) n_part_hyps[p] = (int)lm.size();
        if (part_hyps)
          for (size_t k = 0; k < lm.size(); ++k)
            part_hyp_vect(e, (int)lm[k][0], (int)lm[k][1], (int)lm[k][2], (float)lm[k][3],
                          part_hyps + ((size_t)p * K + k) * 7);
      }
    }
    /* root rotation marginalisation, :694-726 */
    if (e->use_pairwise) {
      std::vector<int> keep;
      if (t->is_upright[root]) {
        int k1 = index_from_rot(e, -1e-6), k2 = index_from_rot(e, 1e-6);
        keep.push_back(k1);
        if (k2 != k1) keep.push_back(k2);
      } else {
        for (int r = 0; r < R; ++r) keep.push_back(r);
      }
      T *rp = root_full.data() + (size_t)sc * HW;
      const T *pr = post[root].data();
      for (size_t i = 0; i < HW; ++i) rp[i] = Num<T>::ex(pr[keep[0] * HW + i]);
      for (size_t k = 1; k < keep.size(); ++k)
        for (size_t i = 0; i < HW; ++i) rp[i] = rp[i] + Num<T>::ex(pr[keep[k] * HW + i]);
      log_grid(rp, HW);
    }
  }

  if (e->use_pairwise && (root_post_out || root_hyps || n_root_hyps)) {
    if (root_post_out) std::copy(root_full.begin(), root_full.end(), root_post_out);
    /* findLocalMax(..., max_hypothesis_number = 1000), :1037-1038 */
    auto lm = find_local_max(root_full.data(), S, H, W, 1000);
    if (n_root_hyps) *n_root_hyps = (int)lm.size();
    if (root_hyps)
      for (size_t k = 0; k < lm.size(); ++k) {
        root_hyps[4 * k + 0] = (float)scale_from_index(e, (int)lm[k][0]);
        root_hyps[4 * k + 1] = (float)lm[k][1];
        root_hyps[4 * k + 2] = (float)lm[k][2];
        root_hyps[4 * k + 3] = (float)lm[k][3];
      }
  } else if (n_root_hyps) {
    *n_root_hyps = 0;
  }
  return 0;
}

/* hc::inverse, libBoostMath/homogeneous_coord.cpp:49-69 */
void hc_inverse(const double *T, double *I) {
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

float eval_stumps(const int32_t *f, const float *p, const float *theta, const float *alpha,
                  int n, float sum_alpha, const float *v, int normalize) {
  float s = 0;
  for (int i = 0; i < n; ++i) {
    const float val = v[f[i]];
    s += (val * p[i] < theta[i] * p[i]) ? alpha[i] : -alpha[i];
  }
  if (normalize) s /= sum_alpha;
  return s;
}

}  // namespace

extern "C" {

void orc_adaboost_eval(const int32_t *f, const float *p, const float *theta, const float *alpha,
                       int n_stumps, float sum_alpha, const float *desc, int64_t n_loc, int D,
                       int normalize, float *out) {
  for (int64_t l = 0; l < n_loc; ++l)
    out[l] = eval_stumps(f, p, theta, alpha, n_stumps, sum_alpha, desc + l * D, normalize);
}

float orc_sum_alpha(const float *alpha, int n_stumps) {
  float s = 0;
  for (int i = 0; i < n_stumps; ++i) s += alpha[i];
  return s;
}

void orc_score_grid_window(const int32_t *f, const float *p, const float *theta,
                           const float *alpha, int n_stumps, float sum_alpha,
                           const float *cells, const uint8_t *valid, int ny, int nx, int Dc,
                           int gx, int gy, double grid_step, int normalize, float *out) {
  std::fill(out, out + (size_t)ny * nx, NO_CLASS_VALUE);
  const int last_ix = nx - bm_round(grid_step * (gx - 1)) - 1;
  const int last_iy = ny - bm_round(grid_step * (gy - 1)) - 1;
  const int D = gx * gy * Dc;
  std::vector<float> v(D);
  for (int iy = 0; iy <= last_iy; ++iy)
    for (int ix = 0; ix <= last_ix; ++ix) {
      bool ok = true;
      for (int ky = 0; ky < gy && ok; ++ky)
        for (int kx = 0; kx < gx && ok; ++kx) {
          int x = ix + bm_round(kx * grid_step), y = iy + bm_round(ky * grid_step);
          if (!valid[(size_t)y * nx + x]) ok = false;
        }
      if (!ok) continue;
      int pos = D;
      for (int ky = 0; ky < gy; ++ky)
        for (int kx = 0; kx < gx; ++kx) {
          int x = ix + bm_round(kx * grid_step), y = iy + bm_round(ky * grid_step);
          pos -= Dc;
          std::memcpy(&v[pos], cells + ((size_t)y * nx + x) * Dc, sizeof(float) * Dc);
        }
      out[(size_t)iy * nx + ix] = eval_stumps(f, p, theta, alpha, n_stumps, sum_alpha, v.data(), normalize);
    }
}

/* The poselet-conditioned extra unaries findObjectImageRotJoints adds before
 * computeRootPosteriorRot (libPictStruct/objectdetect_findrot.cpp:915-948),
 * restated from objectdetect_icps.cpp with the reference's typing:
 * getRotScoreGrid (:228-281) and addExtraUnary (:524-547), getPosScoreGrid
 * (:366-448) and addExtraUnary, setTorsoPosPrior (:137-191).  The grids the
 * reference materialises (log_rot_scores, log_pos_scores: float, zero for
 * the parts they skip; pred_pos: double) are materialised here too.
 * lu: [P][S][R][H][W]. */
int orc_extra_unary(const orc_exp *e, int P, int root, float rot_weight, const double *rot_params,
                    float pos_weight, const double *pos_params, double root_det_x,
                    double root_det_y, float torso_weight, const double *torso_prior,
                    const int *is_detect, float *lu, int S, int H, int W) {
  if (!e || P < 1 || root < 0 || root >= P || !lu || S < 1 || H < 1 || W < 1) return 1;
  const int R = e->num_rotation_steps;
  const size_t HW = (size_t)H * W, N3 = (size_t)R * HW;
  auto detect = [&](int p) { return is_detect ? is_detect[p] != 0 : true; };
  std::vector<float> grid((size_t)P * S * N3);
  if (rot_params) {
    std::fill(grid.begin(), grid.end(), 0.f);
    for (int p = 0; p < P; ++p) {
      if (!detect(p)) continue;
      std::vector<double> pred_rot(R);
      const float mu = (float)rot_params[2 * p];
      const float var = (float)rot_params[2 * p + 1];
      for (int r = 0; r < R; ++r) {
        const float rot = (float)(rot_from_index(e, r) / 180 * M_PI);
        const float d = rot - mu;
        const float sq = d * d;  /* square(), libMisc/misc.hpp:29 */
        float score = (float)std::exp(-0.5 * sq / var);
        if (score < 1e-4) score = (float)1e-4;
        score = std::log(score);
        pred_rot[r] = score;
      }
      for (int s = 0; s < S; ++s)
        for (int r = 0; r < R; ++r)
          for (size_t i = 0; i < HW; ++i)
            grid[((size_t)p * S + s) * N3 + (size_t)r * HW + i] = (float)pred_rot[r];
    }
    for (size_t i = 0; i < grid.size(); ++i) lu[i] += rot_weight * grid[i];
  }
  if (pos_params) {
    std::fill(grid.begin(), grid.end(), 0.f);
    for (int p = 0; p < P; ++p) {
      if (p == root || !detect(p)) continue;
      std::vector<double> pred_pos(HW);
      const float mu_x = (float)pos_params[4 * p], mu_y = (float)pos_params[4 * p + 1];
      const float var_x = (float)(pos_params[4 * p + 2] * 1.0f);
      const float var_y = (float)(pos_params[4 * p + 3] * 1.0f);
      for (int iy = 0; iy < H; ++iy)
        for (int ix = 0; ix < W; ++ix) {
          const float ix_rel = (float)(ix - root_det_x);
          const float iy_rel = (float)(iy - root_det_y);
          const float score_x = (float)std::exp(-0.5 * std::pow((double)(ix_rel - mu_x), 2) / var_x);
          const float score_y = (float)std::exp(-0.5 * std::pow((double)(iy_rel - mu_y), 2) / var_y);
          float score = score_x * score_y;
          if (score < 1e-4) score = (float)1e-4;
          score = std::log(score);
          pred_pos[(size_t)iy * W + ix] = score;
        }
      for (int s = 0; s < S; ++s)
        for (int r = 0; r < R; ++r)
          for (size_t i = 0; i < HW; ++i)
            grid[((size_t)p * S + s) * N3 + (size_t)r * HW + i] = (float)pred_pos[i];
    }
    for (size_t i = 0; i < grid.size(); ++i) lu[i] += pos_weight * grid[i];
  }
  if (torso_prior) {
    const float mu_x = (float)torso_prior[0], mu_y = (float)torso_prior[1];
    float var_x = (float)torso_prior[2], var_y = (float)torso_prior[3];
    const float img_c_x = (float)(0.5 * W), img_c_y = (float)(0.5 * H);
    const float sigma_weight = 1.0f, var_weight = sigma_weight * sigma_weight;
    var_x *= var_weight;
    var_y *= var_weight;
    std::vector<double> pred_pos(HW);
    for (int iy = 0; iy < H; ++iy)
      for (int ix = 0; ix < W; ++ix) {
        const float ix_rel = img_c_x - ix, iy_rel = img_c_y - iy;
        const float score_x = (float)std::exp(-0.5 * std::pow((double)(ix_rel - mu_x), 2) / var_x);
        const float score_y = (float)std::exp(-0.5 * std::pow((double)(iy_rel - mu_y), 2) / var_y);
        float score = torso_weight * score_x * score_y;
        if (score < 1e-4) score = (float)1e-4;
        score = std::log(score);
        pred_pos[(size_t)iy * W + ix] = score;
      }
    for (int s = 0; s < S; ++s)
      for (int r = 0; r < R; ++r)
        for (size_t i = 0; i < HW; ++i) {
          float &c = lu[((size_t)root * S + s) * N3 + (size_t)r * HW + i];
          c = (float)(c + pred_pos[i]);
        }
  }
  return 0;
}

/* The DPM terms of findObjectImageRotJoints, objectdetect_findrot.cpp:883-914,
 * in that order, each a full pass over lu [P][S][R][H][W] as the reference
 * makes it:
 *   torso: computeLogGrid of the torso grid (float), then addDPMScore
 *          (objectdetect_icps.cpp:488-522) on the root part
 *   head:  addLoadDPMScore (:445-486) with pidx_only = head_part, one grid
 *   unary: addLoadDPMScore on every detected part, grids [P][Ru][H][W] with
 *          Ru = R (rotidx_dpm = rotidx) or 1 (rotidx_dpm = 0) */
static void load_dpm_add(float *lu, const float *grid, int Ru, float dpm_weight, int S, int R,
                         size_t HW) {
  for (int s = 0; s < S; ++s)
    for (int r = 0; r < R; ++r) {
      const int rd = (Ru == R ? r : 0);
      for (size_t i = 0; i < HW; ++i) {
        const float val = grid[(size_t)rd * HW + i];
        float &c = lu[((size_t)s * R + r) * HW + i];
        c += (val > 1e-4 ? dpm_weight * std::log(val) : std::log(1e-4));
      }
    }
}

int orc_dpm_score(const orc_exp *e, int P, int root, float torso_weight, const float *torso,
                  float head_weight, int head_part, const float *head, float unary_weight,
                  int unary_rot, const float *unary, const int *is_detect, float *lu, int S,
                  int H, int W) {
  if (!e || P < 1 || root < 0 || root >= P || !lu || S < 1 || H < 1 || W < 1) return 1;
  if (head && (head_part < 0 || head_part >= P)) return 1;
  const int R = e->num_rotation_steps;
  const size_t HW = (size_t)H * W, NP = (size_t)S * R * HW;
  auto detect = [&](int p) { return is_detect ? is_detect[p] != 0 : true; };
  if (torso) {
    std::vector<float> lg(torso, torso + HW);
    log_grid(lg.data(), HW);
    for (int s = 0; s < S; ++s)
      for (int r = 0; r < R; ++r)
        for (size_t i = 0; i < HW; ++i)
          lu[(size_t)root * NP + ((size_t)s * R + r) * HW + i] += torso_weight * lg[i];
  }
  if (head && detect(head_part))
    load_dpm_add(lu + (size_t)head_part * NP, head, 1, head_weight, S, R, HW);
  if (unary) {
    const int Ru = unary_rot ? R : 1;
    for (int p = 0; p < P; ++p)
      if (detect(p)) load_dpm_add(lu + (size_t)p * NP, unary + (size_t)p * Ru * HW, Ru, unary_weight, S, R, HW);
  }
  return 0;
}

/* nms_recursive, libPictStruct/objectdetect_aux.cpp:407-451: hypotheses
 * sorted by descending score (returns 2 when not, where the reference
 * asserts); ellipse_size 0.5, dist_threshold 1.0; the coordinates and scale
 * are the float fields of HypothesisList.proto. */
int orc_nms_recursive(int n, const float *x, const float *y, const float *scale,
                      const float *score, double train_object_width,
                      double train_object_height, int *nms) {
  const double dist_threshold = 1.0, ellipse_size = 0.5;
  if (n < 0) return 1;
  for (int i = 0; i < n; ++i) nms[i] = 0;
  for (int i = 0; i < n; ++i) {
    if (i != n - 1 && score[i] < score[i + 1]) return 2;
    const double sc = scale[i];
    for (int j = i + 1; j < n; ++j) {
      const double a = ellipse_size * sc * train_object_width;
      const double b = ellipse_size * sc * train_object_height;
      const double e1 = a * a, e2 = b * b;
      const double dx = x[i] - x[j];
      const double dy = y[i] - y[j];
      if (dx * dx / e1 + dy * dy / e2 < dist_threshold) nms[j] = 1;
    }
  }
  return 0;
}

/* rect_from_hyp, libNms/nms.cpp:23-56: the upright rectangle (c = 1, s = 0)
 * of a hypothesis, (int)(scale * reference) pixels high and wide, corners
 * p - v1 - v2, p + v1 - v2, p + v1 + v2, p - v1 + v2 in QPointF (double)
 * arithmetic. */
void orc_rect_from_hyp(float x, float y, float scale, double reference_height,
                       double reference_width, double *rect) {
  const int nRectHeight = (int)(scale * reference_height);
  const int nRectWidth = (int)(scale * reference_width);
  const double c = 1, s = 0;
  const double v1x = c * nRectWidth / 2, v1y = s * nRectWidth / 2;
  const double v2x = -s * nRectHeight / 2, v2y = c * nRectHeight / 2;
  const double px = x, py = y;
  rect[0] = px - v1x - v2x, rect[1] = py - v1y - v2y;
  rect[2] = px + v1x - v2x, rect[3] = py + v1y - v2y;
  rect[4] = px + v1x + v2x, rect[5] = py + v1y + v2y;
  rect[6] = px - v1x + v2x, rect[7] = py - v1y + v2y;
}

/* nms_recursive(rects, rect_scores, nms, ellipse_size), libNms/nms.cpp:
 * 132-225 (get_rect_center :126-131): rects [n][4][2], scores descending
 * (returns 2 when not, where the reference asserts); dist_threshold 1.0. */
int orc_nms_rects(int n, const double *rects, const double *scores, double ellipse_size,
                  int *nms) {
  const double dist_threshold = 1.0;
  if (n < 0) return 1;
  for (int i = 0; i < n; ++i) nms[i] = 0;
  auto center = [&](int k, double &cx, double &cy) {
    const double *r = rects + 8 * (size_t)k;
    cx = 0.25 * (r[0] + r[2] + r[4] + r[6]);
    cy = 0.25 * (r[1] + r[3] + r[5] + r[7]);
  };
  for (int i = 0; i < n; ++i) {
    if (i != n - 1 && scores[i] < scores[i + 1]) return 2;
    const double *r = rects + 8 * (size_t)i;
    double v1x = r[2] - r[0], v1y = r[3] - r[1];
    double v2x = r[2] - r[4], v2y = r[3] - r[5];
    const double e1 = v1x * v1x + v1y * v1y;
    const double e2 = v2x * v2x + v2y * v2y;
    const double n1 = std::sqrt(e1), n2 = std::sqrt(e2);
    v1x /= n1, v1y /= n1;
    v2x /= n2, v2y /= n2;
    double c1x, c1y;
    center(i, c1x, c1y);
    for (int j = i + 1; j < n; ++j) {
      double c2x, c2y;
      center(j, c2x, c2y);
      const double px = c2x - c1x, py = c2y - c1y;
      const double dx = v1x * px + v1y * py;
      const double dy = v2x * px + v2y * py;
      if (dx * dx / e1 + dy * dy / e2 < ellipse_size * ellipse_size * dist_threshold) nms[j] = 1;
    }
  }
  return 0;
}

int orc_squeeze_bbox(const float *grid, int ny, int nx, int *bbox) {
  int minx = nx, maxx = -1, miny = ny, maxy = -1;
  for (int ix = 0; ix < nx; ++ix)
    for (int iy = 0; iy < ny; ++iy)
      if (grid[(size_t)iy * nx + ix] != NO_CLASS_VALUE) {
        minx = std::min(minx, ix);
        maxx = std::max(maxx, ix);
        miny = std::min(miny, iy);
        maxy = std::max(maxy, iy);
      }
  bbox[0] = minx;
  bbox[1] = miny;
  bbox[2] = maxx;
  bbox[3] = maxy;
  return (maxx > minx && maxy > miny) ? 1 : 0;
}

void orc_transform_grid(const float *gin, int in_h, int in_w, float *gout, int out_h, int out_w,
                        const double *T21, float def, int method) {
  if (method == 2) { /* TM_DIRECT, multi_array_transform.hpp:173-193 */
    std::fill(gout, gout + (size_t)out_h * out_w, def);
    for (int x1 = 0; x1 < in_w; ++x1)
      for (int y1 = 0; y1 < in_h; ++y1) {
        float v = gin[(size_t)y1 * in_w + x1];
        if (v != def) {
          double x3 = T21[0] * x1 + T21[1] * y1 + T21[2];
          double y3 = T21[3] * x1 + T21[4] * y1 + T21[5];
          int ix3 = (int)std::floor(x3 + 0.5), iy3 = (int)std::floor(y3 + 0.5);
          if (ix3 >= 0 && ix3 < out_w && iy3 >= 0 && iy3 < out_h) gout[(size_t)iy3 * out_w + ix3] = v;
        }
      }
    return;
  }
  double T13[9];
  hc_inverse(T21, T13);
  const float eps10 = 10 * std::numeric_limits<float>::epsilon();
  for (int x3 = 0; x3 < out_w; ++x3)
    for (int y3 = 0; y3 < out_h; ++y3) {
      float o = def;
      double x1 = T13[0] * x3 + T13[1] * y3 + T13[2];
      double y1 = T13[3] * x3 + T13[4] * y3 + T13[5];
      int ix1, iy1;
      if (method == 1) {
        ix1 = (int)std::floor(x1);
        iy1 = (int)std::floor(y1);
      } else {
        ix1 = (int)std::floor(x1 + 0.5);
        iy1 = (int)std::floor(y1 + 0.5);
      }
      if (ix1 >= 0 && ix1 < in_w && iy1 >= 0 && iy1 < in_h) {
        if (method == 0) {
          o = gin[(size_t)iy1 * in_w + ix1];
        } else {
          float a = (float)(x1 - ix1), b = (float)(y1 - iy1);
          if (a < eps10 && b < eps10) {
            o = gin[(size_t)iy1 * in_w + ix1];
          } else if (ix1 < in_w - 1 && iy1 < in_h - 1) {
            const float *g0 = gin + (size_t)iy1 * in_w + ix1, *g1 = g0 + in_w;
            o = (1.0f - b) * (1.0f - a) * g0[0] + (1.0f - b) * a * g0[1] +
                b * (1.0f - a) * g1[0] + b * a * g1[1];
          }
        }
      }
      gout[(size_t)y3 * out_w + x3] = o;
    }
}

void orc_clip_log(float *grid, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (grid[i] < 0) grid[i] = (float)0.0001;
  log_grid(grid, (size_t)n);
}

void orc_eig2d(const double *M, double *V, double *E) { eig2d(M, V, E); }

int orc_gaussian_filter(double sigma, double *out) {
  std::vector<double> f = gaussian_filter(sigma);
  std::copy(f.begin(), f.end(), out);
  return (int)f.size();
}

int orc_rot_joint_marginal_f32(const orc_exp *e, const float *child, float *parent, int R, int H,
                               int W, const double *oc, const double *op, const double *C,
                               double rot_mean, double rot_sigma, double scale) {
  return rot_joint_marginal<float>(e, child, parent, R, H, W, oc, op, C, rot_mean, rot_sigma, scale,
                                   e->sparse_up != 0);
}
int orc_rot_joint_marginal_f64(const orc_exp *e, const double *child, double *parent, int R, int H,
                               int W, const double *oc, const double *op, const double *C,
                               double rot_mean, double rot_sigma, double scale) {
  return rot_joint_marginal<double>(e, child, parent, R, H, W, oc, op, C, rot_mean, rot_sigma, scale,
                                    e->sparse_up != 0);
}

int orc_ps_infer_f32(const orc_exp *e, const orc_tree *t, const float *log_unary, int H, int W,
                     float *log_marg, float *best_conf, float *root_post, float *part_hyps,
                     int *n_part_hyps, float *root_hyps, int *n_root_hyps) {
  return ps_infer<float>(e, t, log_unary, H, W, log_marg, best_conf, root_post, part_hyps,
                         n_part_hyps, root_hyps, n_root_hyps);
}
int orc_ps_infer_f64(const orc_exp *e, const orc_tree *t, const double *log_unary, int H, int W,
                     double *log_marg, float *best_conf, double *root_post, float *part_hyps,
                     int *n_part_hyps, float *root_hyps, int *n_root_hyps) {
  return ps_infer<double>(e, t, log_unary, H, W, log_marg, best_conf, root_post, part_hyps,
                          n_part_hyps, root_hyps, n_root_hyps);
}

int orc_find_local_max(const float *grid, int S, int H, int W, int max_n, double *out) {
  auto lm = find_local_max(grid, S, H, W, max_n);
  for (size_t k = 0; k < lm.size(); ++k)
    for (int c = 0; c < 4; ++c) out[4 * k + c] = lm[k][c];
  return (int)lm.size();
}

int orc_find_obj_f32(const orc_exp *e, const orc_tree *t, const orc_models *m, const float *desc,
                     int ny, int nx, int D, const double *Tig, int interpolate, int H, int W,
                     float *log_unary, float *log_marg, float *best_conf, float *root_post,
                     float *part_hyps, int *n_part_hyps, float *root_hyps, int *n_root_hyps) {
  const int P = t->n_parts, R = e->num_rotation_steps;
  if (m->n_parts < P || n_scales(e) != 1) return -1; /* one scale of descriptors */
  const size_t HW = (size_t)H * W, N = HW * R, G = (size_t)ny * nx;
  std::vector<float> unary((size_t)P * N);
  std::vector<float> grid(G);
  const int S = m->n_stumps;
  /* partdetect_dense scores every loaded classifier; the first P are the
   * part detectors of the tree (partdetect_test.cpp:197-228) */
  for (int p = 0; p < m->n_parts; ++p)
    for (int r = 0; r < R; ++r) {
      orc_adaboost_eval(m->f + (size_t)p * S, m->p + (size_t)p * S, m->theta + (size_t)p * S,
                        m->alpha + (size_t)p * S, S, m->sum_alpha[p], desc + (size_t)r * G * D,
                        (int64_t)G, D, 1, grid.data());
      if (p >= P) continue;
      float *u = unary.data() + (size_t)p * N + (size_t)r * HW;
      orc_transform_grid(grid.data(), ny, nx, u, H, W, Tig, NO_CLASS_VALUE, interpolate ? 1 : 2);
      orc_clip_log(u, (int64_t)HW);
    }
  if (log_unary) std::copy(unary.begin(), unary.end(), log_unary);
  orc_exp ef = *e;
  ef.sparse_up = 1; /* findObjectImageRotJoints: bIsSparse = true (objectdetect_findrot.cpp:740) */
  return ps_infer<float>(&ef, t, unary.data(), H, W, log_marg, best_conf, root_post, part_hyps,
                         n_part_hyps, root_hyps, n_root_hyps);
}

int orc_find_obj_batch_f32(const orc_exp *e, const orc_tree *t, const orc_models *m, int n_img,
                           const float *const *desc, int ny, int nx, int D, const double *Tig,
                           int interpolate, int H, int W, float *best_conf, int n_threads) {
  if (n_threads < 1) n_threads = 1;
  std::vector<int> rcs(n_img, 0);
  std::vector<std::thread> pool;
  for (int w = 0; w < n_threads; ++w)
    pool.emplace_back([&, w]() {
      for (int i = w; i < n_img; i += n_threads)
        rcs[i] = orc_find_obj_f32(e, t, m, desc[i], ny, nx, D, Tig, interpolate, H, W, nullptr,
                                  nullptr, best_conf + (size_t)i * t->n_parts * 7, nullptr,
                                  nullptr, nullptr, nullptr, nullptr);
    });
  for (auto &th : pool) th.join();
  for (int rc : rcs)
    if (rc) return rc;
  return 0;
}

int orc_ps_from_scores_batch_f32(const orc_exp *e, const orc_tree *trees, int n_img,
                                 const float *const *scores, int ny, int nx,
                                 const double *Tig, int interpolate, int H, int W,
                                 float *best_conf, int n_threads) {
  if (n_threads < 1) n_threads = 1;
  if (n_scales(e) != 1) return -1;
  std::vector<int> rcs(n_img, 0);
  std::vector<std::thread> pool;
  for (int w = 0; w < n_threads; ++w)
    pool.emplace_back([&, w]() {
      for (int i = w; i < n_img; i += n_threads) {
        const orc_tree *t = trees + i;
        const int P = t->n_parts, R = e->num_rotation_steps;
        const size_t HW = (size_t)H * W, N = HW * R, G = (size_t)ny * nx;
        std::vector<float> unary((size_t)P * N);
        for (int p = 0; p < P; ++p)
          for (int r = 0; r < R; ++r) {
            float *u = unary.data() + (size_t)p * N + (size_t)r * HW;
            orc_transform_grid(scores[i] + ((size_t)p * R + r) * G, ny, nx, u, H, W, Tig,
                               NO_CLASS_VALUE, interpolate ? 1 : 2);
            orc_clip_log(u, (int64_t)HW);
          }
        orc_exp ef = *e;
        ef.sparse_up = 1; /* findObjectImageRotJoints: bIsSparse = true */
        rcs[i] = ps_infer<float>(&ef, t, unary.data(), H, W, nullptr,
                                 best_conf + (size_t)i * P * 7, nullptr, nullptr, nullptr,
                                 nullptr, nullptr);
      }
    });
  for (auto &th : pool) th.join();
  for (int rc : rcs)
    if (rc) return rc;
  return 0;
}

}  // extern "C"
