// pa_api.cu -- host side of the C-ABI (include/partapp_gb300.h).
//
// Builds, for every call, the device-side descriptors of the pipeline
// (stump tables, unary-map transforms, the message schedule of the tree with
// per-message filter taps and shift tables) in one parameter blob, uploads
// it with a single copy, and launches the kernels of k_*.cu on the context's
// stream.  All host-side parameter math (rotation offsets, Gaussian taps,
// index rounding, matrix inverse) repeats the reference's double-precision
// operations in the same order; this file is compiled with FMA contraction
// off so the host rounds exactly as the reference did.
#include <algorithm>
#include <atomic>
#include <functional>
#include <cmath>
#include <map>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <stdexcept>
#include <tuple>
#include <string>
#include <vector>

#include "pa_internal.cuh"

using namespace pa;

struct pa_classifier {
  int dim = 0;
  int n = 0;
  int npad = 0;
  float sum_alpha = 0.f;
  float4 *d = nullptr;     // {f, p, theta*p, alpha}
  float4 *fast = nullptr;  // {f, t, p*alpha, 0}, only when every p is +1 or -1
  char *packed = nullptr;  // f8[npad/8] (uint4) then ta2[npad/2] (float4)
  std::vector<float4> fast_h;  // host copy of `fast` (rank tables of classifier sets)
  uint64_t id = 0;             // process-unique: the key of cached per-set tables
};

struct pa_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  uint64_t launches = 0;
  char *arena = nullptr;
  size_t arena_cap = 0;
  // pa_find_obj_scales: every scale's unaries [P][S][R][H][W] and one scale's
  // scores and unary maps, kept across the calls that fill the arena
  char *scales_buf = nullptr;
  size_t scales_cap = 0;
  // pinned staging of plan blobs, used round-robin: a buffer is rewritten
  // only after the upload kernel that last read it has run, so a call can
  // plan the next image while the GPU still works on the previous one
  struct Staging {
    char *p = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
  };
  static constexpr int kStages = 4;
  Staging stage[kStages];
  int stage_next = 0;
  // pinned landing blocks of the small per-image results (one per ring slot)
  struct Landing {
    char *p = nullptr;
    size_t cap = 0;
  };
  static constexpr int kLandings = 3;
  std::vector<Landing> land = std::vector<Landing>(kLandings);  // grown by pa_find_obj_queue
  // pa_find_obj_queue: side streams of the per-image work around the queue,
  // pinned status words of the wave in flight
  std::vector<cudaStream_t> side;
  int *qwords = nullptr;
  std::vector<cudaEvent_t> ring_done;  // per ring slot: the slot's image is computed
  // host-input ring: descriptor slots filled on copy_stream while the main
  // stream computes on the previous slot
  cudaStream_t copy_stream = nullptr;
  char *ring = nullptr;
  size_t ring_cap = 0;
  std::vector<cudaEvent_t> ring_ev;
  // per-kernel device timing (CUDA events around each launch)
  bool timing = false;
  struct Pending {
    const char *name;
    cudaEvent_t a, b;
    int n;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  struct Acc {
    double ms = 0;
    uint64_t n = 0;
  };
  std::map<std::string, Acc> times;
  std::vector<std::string> names;  // stable storage for pa_ctx_timing_get
  int msg_math = PA_MSG_FP32;      // spatial filter of diagonal-covariance messages
  // worker contexts (own stream, workspace, staging and landing slots) that
  // run independent image groups of one pa_find_obj_multi call side by side
  static constexpr int kWorkers = 4;
  std::vector<pa_ctx *> workers;
  // pa_find_obj_queue: measured row-tile width per shape class (R, W, kx)
  std::map<std::tuple<int, int, int>, int> row_tile;
  // rank tables of the classifier sets seen (key: the classifiers' ids)
  struct RankEntry {
    bool ok = false;  // false: the set does not qualify (float kernels)
    char *mem = nullptr;
    pa::RankTables rt{};
  };
  std::map<std::vector<uint64_t>, RankEntry> rank_sets;
};

namespace {

pa_status fail(pa_ctx *ctx, pa_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return st;
}

#define PA_CK(call)                                                                 \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(ctx, PA_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));        \
  } while (0)

// Launches `nk` kernels through `call`, timed when the context records
// timing.  Every launch is counted in pa_ctx_kernel_launches.
#define PA_LAUNCH_N(name, nk, call)                                \
  do {                                                             \
    cudaEvent_t ev_a_ = nullptr, ev_b_ = nullptr;                  \
    if (ctx->timing) {                                             \
      ev_a_ = take_event(ctx);                                     \
      ev_b_ = take_event(ctx);                                     \
      cudaEventRecord(ev_a_, ctx->stream);                         \
    }                                                              \
    PA_CK(call);                                                   \
    if (ctx->timing) {                                             \
      cudaEventRecord(ev_b_, ctx->stream);                         \
      ctx->pending.push_back({name, ev_a_, ev_b_, (nk)});          \
    }                                                              \
    ctx->launches += (nk);                                         \
  } while (0)
#define PA_LAUNCH(name, call) PA_LAUNCH_N(name, 1, call)

cudaEvent_t take_event(pa_ctx *ctx) {
  if (!ctx->pool.empty()) {
    cudaEvent_t e = ctx->pool.back();
    ctx->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Called after the stream has been synchronised.
void resolve_timing(pa_ctx *ctx) {
  for (auto &p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      auto &acc = ctx->times[p.name];
      acc.ms += ms;
      acc.n += (uint64_t)p.n;
    } else {
      cudaGetLastError();
    }
    ctx->pool.push_back(p.a);
    ctx->pool.push_back(p.b);
  }
  ctx->pending.clear();
}

pa_status sync_ctx(pa_ctx *ctx) {
  PA_CK(cudaStreamSynchronize(ctx->stream));
  resolve_timing(ctx);
  return PA_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// ------------------------------------------------------------------------
// Two-pass layout builder.  Pass 1 (dry) only measures the parameter blob
// and the device scratch; pass 2 fills the blob with final device pointers.
// The arena holds [parameter blob | scratch].
// ------------------------------------------------------------------------
struct Builder {
  bool dry = true;
  char *base = nullptr;         // device arena (pass 2)
  size_t blob_size = 0;         // pass-2 size of the blob region (from pass 1)
  std::vector<char> blob;
  size_t scratch_off = 0;

  static size_t al(size_t v, size_t a) { return (v + a - 1) / a * a; }

  template <class T>
  T *param(const T *src, size_t n) {
    const size_t o = al(blob.size(), 256);
    blob.resize(o + n * sizeof(T));
    if (n && src) std::memcpy(blob.data() + o, src, n * sizeof(T));
    return dry ? nullptr : reinterpret_cast<T *>(base + o);
  }
  template <class T>
  T *scratch(size_t n) {
    const size_t o = al(scratch_off, 256);
    scratch_off = o + n * sizeof(T);
    return dry ? nullptr : reinterpret_cast<T *>(base + al(blob_size, 256) + o);
  }
  // Pass 1 measures the blob as it grows; pass 2 places scratch after the
  // blob size measured in pass 1.  Both must agree on where scratch starts.
  size_t blob_region() const { return al(dry ? blob.size() : blob_size, 256); }
  size_t total() const { return blob_region() + al(scratch_off, 256) + 256; }
};

pa_status ensure_arena(pa_ctx *ctx, size_t bytes) {
  if (ctx->arena_cap >= bytes) return PA_OK;
  PA_CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->arena) cudaFree(ctx->arena);
  ctx->arena = nullptr;
  ctx->arena_cap = 0;
  size_t cap = bytes + bytes / 8;
  if (cudaMalloc(&ctx->arena, cap) != cudaSuccess) {
    cudaGetLastError();
    ctx->arena = nullptr;
    return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes of device workspace", cap);
  }
  ctx->arena_cap = cap;
  return PA_OK;
}

pa_status upload_blob(pa_ctx *ctx, const Builder &b) {
  // every pointer the plan hands to a kernel lies inside the arena
  if (b.dry || b.blob.size() > b.blob_size ||
      b.blob_region() + Builder::al(b.scratch_off, 256) > ctx->arena_cap)
    return fail(ctx, PA_ERR_INVALID, "internal: plan does not fit the workspace");
  if (b.blob.empty()) return PA_OK;
  pa_ctx::Staging &sg = ctx->stage[ctx->stage_next];
  ctx->stage_next = (ctx->stage_next + 1) % pa_ctx::kStages;
  if (sg.done) PA_CK(cudaEventSynchronize(sg.done));  // its previous upload has been read
  else PA_CK(cudaEventCreateWithFlags(&sg.done, cudaEventDisableTiming));
  if (sg.cap < b.blob.size()) {
    if (sg.p) cudaFreeHost(sg.p);
    sg.p = nullptr;
    sg.cap = 0;
    const size_t cap = b.blob.size() + b.blob.size() / 4 + 4096;
    if (cudaMallocHost(&sg.p, cap) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes of pinned staging", cap);
    }
    sg.cap = cap;
  }
  std::memcpy(sg.p, b.blob.data(), b.blob.size());
  // a kernel reads the pinned staging buffer directly: the parameters do not
  // queue behind large host->device copies on the copy engines
  PA_LAUNCH("upload", launch_copy16(sg.p, ctx->arena, (int64_t)((b.blob.size() + 15) / 16),
                                    ctx->stream));
  PA_CK(cudaEventRecord(sg.done, ctx->stream));
  return PA_OK;
}

// Host bytes -> a device location through the pinned staging ring and a copy
// kernel (stream-ordered, no host synchronisation); bytes a multiple of 16.
pa_status upload_to(pa_ctx *ctx, void *dst, const void *src, size_t bytes) {
  if (!bytes) return PA_OK;
  pa_ctx::Staging &sg = ctx->stage[ctx->stage_next];
  ctx->stage_next = (ctx->stage_next + 1) % pa_ctx::kStages;
  if (sg.done) PA_CK(cudaEventSynchronize(sg.done));
  else PA_CK(cudaEventCreateWithFlags(&sg.done, cudaEventDisableTiming));
  if (sg.cap < bytes) {
    if (sg.p) cudaFreeHost(sg.p);
    sg.p = nullptr;
    sg.cap = 0;
    if (cudaMallocHost(&sg.p, bytes + 4096) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes of pinned staging", bytes);
    }
    sg.cap = bytes + 4096;
  }
  std::memcpy(sg.p, src, bytes);
  PA_LAUNCH("upload", launch_copy16(sg.p, dst, (int64_t)((bytes + 15) / 16), ctx->stream));
  PA_CK(cudaEventRecord(sg.done, ctx->stream));
  return PA_OK;
}

pa_status copy_in(pa_ctx *ctx, void *dst, const void *src, size_t bytes, int mem) {
  if (!bytes) return PA_OK;
  PA_CK(cudaMemcpyAsync(dst, src, bytes,
                        mem == PA_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                        ctx->stream));
  return PA_OK;
}

// ------------------------------------------------------------------------
// Reference parameter math (host, double precision, reference op order).
// ------------------------------------------------------------------------
double value_from_index(double minval, double maxval, double num_steps, int idx) {
  if (minval == maxval) return minval;                 // partapp_aux.hpp:45-58
  double step_size = (maxval - minval) / num_steps;
  return minval + step_size * (0.5 + idx);
}
int index_from_value(double minval, double maxval, double num_steps, double val) {
  if (minval == maxval) return 0;                      // partapp_aux.hpp:23-43
  double step_size = (maxval - minval) / num_steps;
  return (int)std::floor((val - minval) / step_size);
}
double rot_from_index(const pa_exp_param *e, int idx) {
  return value_from_index(e->min_part_rotation, e->max_part_rotation,
                          (double)(unsigned)e->num_rotation_steps, idx);
}
int index_from_rot(const pa_exp_param *e, double rot) {
  return index_from_value(e->min_part_rotation, e->max_part_rotation,
                          (double)(unsigned)e->num_rotation_steps, rot);
}
// ExpParam::num_scale_steps (ExpParam.proto:191); 0 reads as 1
int n_scales(const pa_exp_param *e) { return e->num_scale_steps > 1 ? e->num_scale_steps : 1; }
double scale_from_index(const pa_exp_param *e, int idx) {
  return value_from_index(e->min_object_scale, e->max_object_scale, (double)n_scales(e), idx);
}

// rotation bin width in radians, objectdetect_findrot.cpp:319-321
double rot_step_rad(const pa_exp_param *e) {
  float step_f = (e->max_part_rotation - e->min_part_rotation) /
                 (float)(unsigned)e->num_rotation_steps;
  double s = step_f;
  s *= M_PI / 180.0;
  return s;
}

// get_gaussian_filter, boost_math.cpp:104-117 (unnormalised)
std::vector<double> gaussian_taps(double sigma) {
  // the same sigmas recur across the images and calls of a model: the taps
  // are kept per host thread, keyed by sigma's bits (cleared past 4096)
  thread_local std::map<uint64_t, std::vector<double>> memo;
  uint64_t key;
  std::memcpy(&key, &sigma, sizeof key);
  auto it = memo.find(key);
  if (it != memo.end()) return it->second;
  int ksize = (int)std::floor(3 * sigma + 0.5);
  std::vector<double> f(2 * ksize + 1);
  f[ksize] = 1.0;
  for (int i = 1; i <= ksize; ++i) {
    f[ksize + i] = std::exp(-i * i / (2 * sigma * sigma));
    f[ksize - i] = f[ksize + i];
  }
  if (memo.size() >= 4096) memo.clear();
  memo.emplace(key, f);
  return f;
}

// prod(prod(R(alpha), S(scale)), (ox, oy, 0)), objectdetect_findrot.cpp:348-351
// cos and sin of the float angle of every rotation bin, kept per host thread
// for the last rotation set seen (a plan rotates two offsets per message and
// rotation bin: ~7000 pairs for 4 images at R = 24).
const std::vector<std::pair<double, double>> &rotation_trig(const pa_exp_param *e) {
  thread_local int n = -1;
  thread_local float lo = 0.f, hi = 0.f;
  thread_local std::vector<std::pair<double, double>> tab;
  if (n != e->num_rotation_steps || lo != e->min_part_rotation || hi != e->max_part_rotation) {
    n = e->num_rotation_steps;
    lo = e->min_part_rotation;
    hi = e->max_part_rotation;
    tab.resize(n > 0 ? n : 0);
    for (int r = 0; r < n; ++r) {
      const float alpha = (float)(rot_from_index(e, r) * M_PI / 180.0);
      tab[r] = {std::cos((double)alpha), std::sin((double)alpha)};
    }
  }
  return tab;
}

void rotate_offset(const pa_exp_param *e, int r, double scale, const double *o, double &dx,
                   double &dy) {
  const auto &cs = rotation_trig(e)[r];
  const double ca = cs.first, sa = cs.second;
  double t00 = ca * scale, t01 = (-sa) * scale;
  double t10 = sa * scale, t11 = ca * scale;
  dx = t00 * o[0] + t01 * o[1];
  dy = t10 * o[0] + t11 * o[1];
}

// hc::inverse, homogeneous_coord.cpp:49-69
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

// The covariances eig2d and gaussFilterDiag2d accept: symmetric, positive
// definite (both eigenvalues > 0).
bool cov_ok(const double *C) {
  if (!(std::isfinite(C[0]) && std::isfinite(C[1]) && std::isfinite(C[2]) && std::isfinite(C[3])))
    return false;
  if (C[1] != C[2]) return false;
  return C[0] > 0 && C[3] > 0 && C[0] * C[3] - C[1] * C[2] > 0;
}

bool exp_ok(const pa_exp_param *e) {
  return e && e->num_rotation_steps >= 2 && e->num_rotation_steps <= kMaxRot &&
         e->max_part_rotation > e->min_part_rotation &&
         e->strip_border_detections >= 0 && e->strip_border_detections < 0.5f &&
         e->roi_save_num_samples >= 0 && e->roi_save_num_samples <= 2048 &&
         e->num_scale_steps >= 0 && e->num_scale_steps <= 64 &&
         // value_from_index asserts one step when min == max (partapp_aux.hpp:48-52)
         (n_scales(e) == 1 || e->max_object_scale > e->min_object_scale);
}

// ------------------------------------------------------------------------
// Tree schedule (computeRootPosteriorRot / computePartMarginals order).
// ------------------------------------------------------------------------
struct Joint {
  double oc[2], op[2], C[4], rot_mean, rot_sigma;
};

struct Sched {
  int P = 0, root = 0, maxdepth = 0;
  std::vector<std::vector<int>> ch, chj;  // children per part, joint order
  std::vector<int> pj, depth, rslot;      // parent joint, depth, slot among root children
  std::vector<int> upright;
};

pa_status build_sched(pa_ctx *ctx, const pa_tree *t, Sched &s) {
  if (!t || t->n_parts < 1 || t->root < 0 || t->root >= t->n_parts)
    return fail(ctx, PA_ERR_INVALID, "invalid tree: n_parts/root");
  const int P = t->n_parts;
  if (t->n_joints != P - 1)
    return fail(ctx, PA_ERR_INVALID, "tree needs n_parts-1 joints (loadJoints asserts this)");
  s.P = P;
  s.root = t->root;
  s.ch.assign(P, {});
  s.chj.assign(P, {});
  s.pj.assign(P, -1);
  s.depth.assign(P, -1);
  s.rslot.assign(P, -1);
  s.upright.assign(P, 0);
  for (int p = 0; p < P; ++p) s.upright[p] = t->is_upright ? (t->is_upright[p] != 0) : 0;
  for (int j = 0; j < t->n_joints; ++j) {
    const int c = t->child[j], q = t->parent[j];
    if (c < 0 || c >= P || q < 0 || q >= P || c == q)
      return fail(ctx, PA_ERR_INVALID, "joint %d: part index out of range", j);
    if (s.pj[c] >= 0 || c == t->root)
      return fail(ctx, PA_ERR_INVALID, "joint %d: part %d has two parents", j, c);
    s.pj[c] = j;
    s.ch[q].push_back(c);
    s.chj[q].push_back(j);
  }
  s.depth[s.root] = 0;
  std::vector<int> order{s.root};
  for (size_t i = 0; i < order.size(); ++i)
    for (int c : s.ch[order[i]]) {
      s.depth[c] = s.depth[order[i]] + 1;
      s.maxdepth = std::max(s.maxdepth, s.depth[c]);
      order.push_back(c);
    }
  if ((int)order.size() != P) return fail(ctx, PA_ERR_INVALID, "joints do not form a tree");
  for (int p = 0; p < P; ++p)
    if (p != s.root && s.ch[p].size() > 1)
      return fail(ctx, PA_ERR_UNSUPPORTED,
                  "part %d has %zu children; the reference supports one child below the root",
                  p, s.ch[p].size());
  if ((int)s.ch[s.root].size() > kMaxRootChildren)
    return fail(ctx, PA_ERR_UNSUPPORTED, "root has more than %d children", kMaxRootChildren);
  for (size_t i = 0; i < s.ch[s.root].size(); ++i) s.rslot[s.ch[s.root][i]] = (int)i;
  return PA_OK;
}

bool same_topology(const pa_tree *a, const pa_tree *b) {
  if (a->n_parts != b->n_parts || a->root != b->root || a->n_joints != b->n_joints) return false;
  for (int j = 0; j < a->n_joints; ++j)
    if (a->child[j] != b->child[j] || a->parent[j] != b->parent[j]) return false;
  for (int p = 0; p < a->n_parts; ++p) {
    const int ua = a->is_upright ? a->is_upright[p] != 0 : 0;
    const int ub = b->is_upright ? b->is_upright[p] != 0 : 0;
    if (ua != ub) return false;
  }
  return true;
}

pa_status load_joints(pa_ctx *ctx, const pa_tree *t, int flip, std::vector<Joint> &js) {
  js.resize(t->n_joints);
  for (int j = 0; j < t->n_joints; ++j) {
    Joint &J = js[j];
    for (int k = 0; k < 2; ++k) {
      J.oc[k] = t->offset_c[2 * j + k];
      J.op[k] = t->offset_p[2 * j + k];
    }
    for (int k = 0; k < 4; ++k) J.C[k] = t->C[4 * j + k];
    J.rot_mean = t->rot_mean[j];
    J.rot_sigma = t->rot_sigma[j];
    if (flip) {  // loadJoints, objectdetect_aux.cpp:98-116
      J.oc[0] = -J.oc[0];
      J.op[0] = -J.op[0];
      J.C[1] = -J.C[1];
      J.C[2] = -J.C[2];
      J.rot_mean = -J.rot_mean;
    }
    if (!cov_ok(J.C))
      return fail(ctx, PA_ERR_INVALID, "joint %d: covariance must be symmetric positive definite", j);
    if (!(std::isfinite(J.rot_mean) && std::isfinite(J.rot_sigma)))
      return fail(ctx, PA_ERR_INVALID, "joint %d: rotation parameters not finite", j);
  }
  return PA_OK;
}

}  // namespace

namespace pa {

// Per-message host parameters of computeRotJointMarginal(child -> parent,
// offset_c_10 = oc, offset_p_01 = op, rot_mean, rot_sigma).

// boost_math::eig2d (libBoostMath/boost_math.cpp:40-99): E = (smallest,
// largest) eigenvalue, V (row-major) holds the eigenvectors as columns.
void eig2d(const double *M, double *V, double *E) {
  const double m11 = M[0], m12 = M[1], m22 = M[3];
  double e1, e2, v11, v21;
  if (m12 != 0) {
    const double sqrtD = std::sqrt((m11 - m22) * (m11 - m22) + 4 * m12 * m12);
    e1 = 0.5 * (m11 + m22 - sqrtD);
    e2 = 0.5 * (m11 + m22 + sqrtD);
    v11 = 0.5 * (m11 - m22 - sqrtD) / m12;
    v21 = 1;
  } else if (m11 < m22) {
    e1 = m11; e2 = m22; v11 = 1; v21 = 0;
  } else {
    e1 = m22; e2 = m11; v11 = 0; v21 = 1;
  }
  const double norm_v1 = std::sqrt(v11 * v11 + v21 * v21);
  v11 /= norm_v1;
  v21 /= norm_v1;
  V[0] = v11;
  V[1] = -v21;
  V[2] = v21;
  V[3] = v11;
  E[0] = e1;
  E[1] = e2;
}

// ublas prod of 3x3 matrices (row-major), accumulated k = 0, 1, 2.
void prod3(const double *A, const double *B, double *Cm) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double t = 0;
      for (int k = 0; k < 3; ++k) t += A[3 * i + k] * B[3 * k + j];
      Cm[3 * i + j] = t;
    }
}

// The transforms of gaussFilter2dOffset with a zero offset
// (libMultiArray/multi_array_filter.hpp:335-369): rotate the [H][W] map into
// the eigenbasis of C (transform_grid_resize, adaptive size from
// hc::get_transformed_bbox, homogeneous_coord.cpp:140-156), filter along the
// eigen axes, rotate back (transform_grid_fixed_size).
void full_cov_params(const double *Cs, int H, int W, bool sparse, MsgParams &m, double *E) {
  double V[4];
  eig2d(Cs, V, E);
  const double T21[9] = {V[0], V[2], 0, V[1], V[3], 0, 0, 0, 1};  // [trans(V) | 0]
  const double px[4] = {0, (double)(W - 1), 0, (double)(W - 1)};
  const double py[4] = {0, 0, (double)(H - 1), (double)(H - 1)};
  double xs[4], ys[4];
  for (int c = 0; c < 4; ++c) {
    xs[c] = T21[0] * px[c] + T21[1] * py[c] + T21[2] * 1.0;
    ys[c] = T21[3] * px[c] + T21[4] * py[c] + T21[5] * 1.0;
  }
  const double minx = *std::min_element(xs, xs + 4), maxx = *std::max_element(xs, xs + 4);
  const double miny = *std::min_element(ys, ys + 4), maxy = *std::max_element(ys, ys + 4);
  m.ow = (int)std::ceil(maxx - minx);
  m.oh = (int)std::ceil(maxy - miny);
  const double T23[9] = {1, 0, minx, 0, 1, miny, 0, 0, 1};
  double T12[9], T13[9];
  hc_inverse(T21, T12);
  prod3(T12, T23, T13);
  const double mz = -0.0;
  const double T42[9] = {V[0], V[1], mz, V[2], V[3], mz, 0, 0, 1};
  double T43[9], Tb[9], Tbb[9];
  prod3(T42, T23, T43);
  hc_inverse(T43, Tb);
  const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  prod3(Tb, I3, Tbb);
  // TM_DIRECT (bIsSparse): input cell -> output cell, T31 = T32 * T21
  const double T32[9] = {1, 0, -minx, 0, 1, -miny, 0, 0, 1};
  double T31[9];
  prod3(T32, T21, T31);
  for (int k = 0; k < 6; ++k) {
    m.tf[k] = T13[k];
    m.tb[k] = Tbb[k];
    m.td[k] = T31[k];
  }
  m.full = true;
  m.sparse = sparse;
}

void msg_params(const pa_exp_param *e, double scale, const double *oc, const double *op,
                const double *C, double rot_mean, double rot_sigma, int H, int W, bool sparse,
                MsgParams &m) {
  const int R = e->num_rotation_steps;
  const double step = rot_step_rad(e);
  const double rot_sigma_idx = rot_sigma / step;
  m.kidx = (int)std::floor(-rot_mean / step + 0.5);
  m.rtaps.clear();
  if (rot_sigma > 0) {  // objectdetect_findrot.cpp:377-404
    std::vector<double> f = gaussian_taps(rot_sigma_idx);
    int first = 0, fs = (int)f.size();
    if (fs >= R) {
      int crot = fs / 2;
      fs = (R % 2 == 1) ? R - 2 : R - 1;
      first = crot - fs / 2;
    }
    for (int i = first; i < first + fs; ++i) m.rtaps.push_back((float)f[i]);
    m.rlen = fs;
  } else if (rot_sigma == 0) {
    m.rlen = -1;
  } else {
    m.rlen = 0;
  }
  const double sc2 = scale * scale;  // gaussFilterDiag2d, multi_array_filter.hpp:232-236
  const double Cs[4] = {sc2 * C[0], sc2 * C[1], sc2 * C[2], sc2 * C[3]};  // square(scale)*C
  double sx2 = Cs[0], sy2 = Cs[3];
  m.full = false;
  m.sparse = false;
  if (Cs[1] != 0 || Cs[2] != 0) {  // gaussFilter2d -> gaussFilter2dOffset
    double E[2];
    full_cov_params(Cs, H, W, sparse, m, E);
    sx2 = E[0];
    sy2 = E[1];
  }
  std::vector<double> fx = gaussian_taps(std::sqrt(sx2));
  std::vector<double> fy = gaussian_taps(std::sqrt(sy2));
  m.xtaps.assign(fx.begin(), fx.end());
  m.ytaps.assign(fy.begin(), fy.end());
  m.xlen = (int)fx.size();
  m.ylen = (int)fy.size();
  m.shifts.assign(4 * (size_t)R, 0.0);
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int r = 0; r < R; ++r) {
    const int rs = r - m.kidx;
    if (rs >= 0 && rs < R) {
      double dx, dy;
      rotate_offset(e, rs, scale, oc, dx, dy);
      m.shifts[0 * R + r] = -dx;
      m.shifts[1 * R + r] = -dy;
    } else {
      m.shifts[0 * R + r] = nan;
      m.shifts[1 * R + r] = nan;
    }
    double dx, dy;
    rotate_offset(e, r, scale, op, dx, dy);
    m.shifts[2 * R + r] = dx;
    m.shifts[3 * R + r] = dy;
  }
}

}  // namespace pa

namespace {

// ------------------------------------------------------------------------
// PS plan for a batch of images (shared topology and sizes).
// ------------------------------------------------------------------------
struct ImgMaps {
  std::vector<float *> U, POST, MARG, TMP, MSGR, FR;
  float *root_post = nullptr;
};

struct PsPlan {
  int B = 0, P = 0, R = 0, H = 0, W = 0;
  int64_t N = 0;
  Sched sc;
  std::vector<ImgMaps> im;
  int *umax = nullptr, *pmax = nullptr, *frmax = nullptr, *tmax = nullptr;  // [B][P]
  unsigned long long *amax = nullptr;                                         // [B][P]
  double *msgmax = nullptr;                                                   // [B][2(P-1)]
  double *logz = nullptr;                                                     // [B][P]
  void *logz_part = nullptr;  // log_z_scratch_bytes(B * P)
  int *err = nullptr;
  struct Phase {
    MsgDesc *msgs = nullptr;
    int n = 0, padx = 0, pady = 0;
    bool tma = false;  // every message of the phase has TMA maps for the column pass
    // per message (host): image, child part, x / y kernel half-widths
    std::vector<int> m_img, m_child, m_kx, m_ky;
    int n_full = 0, ohmax = 0, owmax = 0, kxf = 0, kyf = 0;  // full-covariance messages
    struct TcJob {
      void *eb, *xt, *tbx, *tby;
      float *yv;
      int kx, ky;
    };
    std::vector<TcJob> tc;  // tensor-core messages
  };
  bool tc_mode = false;  // diagonal-covariance messages on the tensor cores (H % 8 == 0)
  bool own_e2 = false;   // every message its own e2 buffer (messages of different
                         // phases in flight together: the persistent queue)
  bool sparse_up = false;  // bIsSparse of the upward messages
  // multi-scale computeRootPosteriorRot: batch entry i is scale img_scale[i]
  // (empty: every entry at scale 0)
  std::vector<int> img_scale;
  int64_t out_pstride = 0;  // elements between the parts of a log_marg output (0: N)
  int hyp_img = -1;         // >= 0: part local maxima of this entry only
  bool root_joint = false;  // root local maxima over [B][H][W] with B as the scale axis
  int wp = 0, hp = 0;
  std::vector<Phase> up, down;
  RootDesc *roots = nullptr;
  int16_t *tables = nullptr;
  int4 *sdesc = nullptr;
  double *shifts = nullptr;
  int n_msgs_total = 0;
  const float **marg_ptrs = nullptr;
  const float **post_root_ptrs = nullptr;
  float **root_post_ptrs = nullptr;
  int *keep = nullptr;
  int n_keep = 0;
  // findLocalMax outputs (objectdetect_aux.cpp:193-320)
  bool want_part_hyps = false, want_root_hyps = false;
  int hyp_k = 0;
  void *lm_scratch = nullptr;
  float *part_hyps = nullptr;   // [B*P][hyp_k][4] (s, x, y, value)
  int *n_part_hyps = nullptr;   // [B*P]
  float *root_hyps = nullptr;   // [B][1000][4]
  int *n_root_hyps = nullptr;   // [B]
};

constexpr int kRootHyps = 1000;  // max_hypothesis_number, objectdetect_findrot.cpp:1037

// Builds the device-side plan.  unary maps U are scratch unless `unary_in`
// gives their final location.  marg_out/root_post_out: per image device
// outputs (nullptr -> scratch).
void plan_ps(Builder &b, PsPlan &pl, const pa_exp_param *e,
             const std::vector<std::vector<Joint>> &joints, float *const *marg_out,
             float *const *root_post_out) {
  const int B = pl.B, P = pl.P, R = pl.R, H = pl.H, W = pl.W;
  const int64_t N = pl.N;
  const Sched &s = pl.sc;
  const int64_t pstride = pl.out_pstride ? pl.out_pstride : N;
  auto scale_of = [&](int img) {
    return scale_from_index(e, pl.img_scale.empty() ? 0 : pl.img_scale[img]);
  };
  pl.im.assign(B, {});
  for (int i = 0; i < B; ++i) {
    ImgMaps &m = pl.im[i];
    m.U.assign(P, nullptr);
    m.POST.assign(P, nullptr);
    m.MARG.assign(P, nullptr);
    m.TMP.assign(P, nullptr);
    m.MSGR.assign(s.ch[s.root].size(), nullptr);
    m.FR.assign(s.ch[s.root].size(), nullptr);
    for (int p = 0; p < P; ++p) {
      m.U[p] = b.scratch<float>(N);
      const bool inner = (p != s.root && !s.ch[p].empty());
      m.POST[p] = inner ? b.scratch<float>(N) : m.U[p];
      m.TMP[p] = inner ? b.scratch<float>(N) : nullptr;
      m.MARG[p] = marg_out && marg_out[i] ? marg_out[i] + (int64_t)p * pstride : b.scratch<float>(N);
    }
    m.POST[s.root] = m.MARG[s.root];
    for (size_t k = 0; k < m.MSGR.size(); ++k) {
      m.MSGR[k] = b.scratch<float>(N);
      m.FR[k] = b.scratch<float>(N);
    }
    m.root_post = root_post_out && root_post_out[i] ? root_post_out[i]
                                                    : b.scratch<float>((size_t)H * W);
  }
  pl.umax = b.scratch<int>((size_t)B * P);
  pl.pmax = b.scratch<int>((size_t)B * P);
  pl.frmax = b.scratch<int>((size_t)B * P);
  pl.tmax = b.scratch<int>((size_t)B * P);
  pl.amax = b.scratch<unsigned long long>((size_t)B * P);
  pl.msgmax = b.scratch<double>((size_t)B * 2 * std::max(1, P - 1));
  pl.logz = b.scratch<double>((size_t)B * P);
  pl.logz_part = b.scratch<double>((log_z_scratch_bytes(B * P) + 7) / 8);
  pl.err = b.scratch<int>(1);

  if (!e->use_pairwise) return;

  // message list: upward by decreasing depth, downward by increasing depth
  struct M {
    int img, child, parent, joint;
    bool up;
  };
  std::vector<std::vector<M>> upph, dnph;
  std::vector<int> parent_of(P, -1);
  for (int p = 0; p < P; ++p)
    for (int c : s.ch[p]) parent_of[c] = p;
  for (int d = s.maxdepth; d >= 1; --d) {
    std::vector<M> ph;
    for (int i = 0; i < B; ++i)
      for (int c = 0; c < P; ++c)
        if (s.depth[c] == d) ph.push_back({i, c, parent_of[c], s.pj[c], true});
    upph.push_back(ph);
  }
  for (int d = 1; d <= s.maxdepth; ++d) {
    std::vector<M> ph;
    for (int i = 0; i < B; ++i)
      for (int c = 0; c < P; ++c)
        if (s.depth[c] == d) ph.push_back({i, c, parent_of[c], s.pj[c], false});
    dnph.push_back(ph);
  }
  size_t maxph = 0;
  for (auto &ph : upph) maxph = std::max(maxph, ph.size());
  for (auto &ph : dnph) maxph = std::max(maxph, ph.size());
  std::vector<float *> e2(pl.own_e2 ? 0 : maxph);
  for (size_t k = 0; k < e2.size(); ++k) e2[k] = b.scratch<float>(N);
  // message parameters; rotated-grid buffers of full-covariance messages are
  // shared by the messages that take slot k in their phase
  auto params_of = [&](const M &mm) {
    const Joint &J = joints[mm.img][mm.joint];
    MsgParams mp;
    // upward messages take the caller's bIsSparse (objectdetect_findrot.cpp:630-635),
    // downward ones are dense (:174-179, 224-229)
    const double scale = scale_of(mm.img);
    if (mm.up)
      msg_params(e, scale, J.oc, J.op, J.C, J.rot_mean, J.rot_sigma, H, W, pl.sparse_up, mp);
    else
      msg_params(e, scale, J.op, J.oc, J.C, -J.rot_mean, J.rot_sigma, H, W, false, mp);
    return mp;
  };
  std::vector<std::vector<MsgParams>> upmp(upph.size()), dnmp(dnph.size());
  std::vector<size_t> slot_cells(maxph, 0);
  for (size_t k = 0; k < upph.size(); ++k)
    for (const M &mm : upph[k]) upmp[k].push_back(params_of(mm));
  for (size_t k = 0; k < dnph.size(); ++k)
    for (const M &mm : dnph[k]) dnmp[k].push_back(params_of(mm));
  for (auto *all : {&upmp, &dnmp})
    for (auto &v : *all)
      for (size_t k = 0; k < v.size(); ++k)
        if (v[k].full) slot_cells[k] = std::max(slot_cells[k], (size_t)v[k].oh * v[k].ow);
  std::vector<float *> g0(maxph, nullptr), g1(maxph, nullptr);
  for (size_t k = 0; k < maxph; ++k)
    if (slot_cells[k]) {
      g0[k] = b.scratch<float>((size_t)R * slot_cells[k]);
      g1[k] = b.scratch<float>((size_t)R * slot_cells[k]);
    }
  // tensor-core messages: bf16 operands and the fp32 y-pass result per slot
  const bool tc = pl.tc_mode && (H % 8) == 0;
  pl.wp = (W + 7) / 8 * 8;
  pl.hp = (H + 7) / 8 * 8;
  std::vector<bool> slot_tc(maxph, false);
  for (auto *all : {&upmp, &dnmp})
    for (auto &v : *all)
      for (size_t k = 0; k < v.size(); ++k)
        if (tc && !v[k].full) slot_tc[k] = true;
  struct TcBufs {
    uint16_t *eb = nullptr, *xt = nullptr, *tbx = nullptr, *tby = nullptr;
    float *yv = nullptr;
  };
  std::vector<TcBufs> tcb(maxph);
  for (size_t k = 0; k < maxph; ++k)
    if (slot_tc[k]) {
      tcb[k].eb = b.scratch<uint16_t>((size_t)R * H * pl.wp);
      tcb[k].xt = b.scratch<uint16_t>((size_t)W * R * H);
      tcb[k].tbx = b.scratch<uint16_t>((size_t)W * pl.wp);
      tcb[k].tby = b.scratch<uint16_t>((size_t)H * pl.hp);
      tcb[k].yv = b.scratch<float>((size_t)R * H * W);
    }

  pl.n_msgs_total = 0;
  for (auto &ph : upph) pl.n_msgs_total += (int)ph.size();
  for (auto &ph : dnph) pl.n_msgs_total += (int)ph.size();
  const size_t tbl_per = (size_t)2 * R * (W + H);
  std::vector<double> all_shifts;
  all_shifts.reserve((size_t)pl.n_msgs_total * 4 * R);

  int msg_counter = 0;
  auto build_phase = [&](const std::vector<M> &ph, const std::vector<MsgParams> &mps,
                         PsPlan::Phase &out) {
    std::vector<MsgDesc> descs(ph.size());
    out.n = (int)ph.size();
    out.m_img.clear();
    out.m_child.clear();
    out.m_kx.clear();
    out.m_ky.clear();
    out.padx = out.pady = 0;
    out.tc.clear();
    for (size_t k = 0; k < ph.size(); ++k) {
      const M &mm = ph[k];
      const int c = mm.child;
      const int par = mm.parent;
      const MsgParams &mp = mps[k];
      ImgMaps &im = pl.im[mm.img];
      MsgDesc &d = descs[k];
      std::memset(&d, 0, sizeof d);
      const int ib = mm.img * P;
      const int gidx = msg_counter++;
      const size_t toff = (size_t)gidx * tbl_per;
      d.tx_in = b.dry ? nullptr : pl.tables + toff;
      d.ty_in = b.dry ? nullptr : pl.tables + toff + (size_t)R * W;
      d.tx_out = b.dry ? nullptr : pl.tables + toff + (size_t)R * (W + H);
      d.ty_out = b.dry ? nullptr : pl.tables + toff + (size_t)R * (W + H) + (size_t)R * W;
      d.sdesc = b.dry ? nullptr : pl.sdesc + (size_t)gidx * 4 * R;
      all_shifts.insert(all_shifts.end(), mp.shifts.begin(), mp.shifts.end());
      d.rtaps = mp.rtaps.empty() ? nullptr : b.param(mp.rtaps.data(), mp.rtaps.size());
      d.xtaps = b.param(mp.xtaps.data(), mp.xtaps.size());
      d.ytaps = b.param(mp.ytaps.data(), mp.ytaps.size());
      d.kidx = mp.kidx;
      d.rlen = mp.rlen;
      d.xlen = mp.xlen;
      d.ylen = mp.ylen;
      d.e2 = pl.own_e2 ? b.scratch<float>(N) : e2[k];
      out.m_img.push_back(mm.img);
      out.m_child.push_back(c);
      out.m_kx.push_back((mp.xlen - 1) / 2);
      out.m_ky.push_back((mp.ylen - 1) / 2);
      if (mp.full) {
        d.full = 1;
        d.oh = mp.oh;
        d.ow = mp.ow;
        d.g0 = g0[k];
        d.g1 = g1[k];
        for (int q = 0; q < 6; ++q) {
          d.tf[q] = mp.tf[q];
          d.tb[q] = mp.tb[q];
          d.td[q] = mp.td[q];
        }
        d.sparse = mp.sparse ? 1 : 0;
        ++out.n_full;
        out.ohmax = std::max(out.ohmax, mp.oh);
        out.owmax = std::max(out.owmax, mp.ow);
        out.kxf = std::max(out.kxf, (mp.xlen - 1) / 2);
        out.kyf = std::max(out.kyf, (mp.ylen - 1) / 2);
      } else if (slot_tc[k]) {
        d.tc = 1;
        d.wp = pl.wp;
        d.hp = pl.hp;
        d.eb = tcb[k].eb;
        d.xt = tcb[k].xt;
        d.tbx = tcb[k].tbx;
        d.tby = tcb[k].tby;
        d.yv = tcb[k].yv;
        out.tc.push_back({tcb[k].eb, tcb[k].xt, tcb[k].tbx, tcb[k].tby, tcb[k].yv,
                          (mp.xlen - 1) / 2, (mp.ylen - 1) / 2});
      } else {
        out.padx = std::max(out.padx, (mp.xlen - 1) / 2);
        out.pady = std::max(out.pady, (mp.ylen - 1) / 2);
      }
      if (mm.up) {
        const bool inner = !s.ch[c].empty();
        d.in = inner ? im.POST[c] : im.U[c];
        d.in_max = b.dry ? nullptr : (inner ? pl.pmax : pl.umax) + ib + c;
        if (par == s.root) {
          d.mode = EPI_STORE;
          d.dst0 = im.MSGR[s.rslot[c]];
        } else {
          d.mode = EPI_ADD;
          d.dst0 = im.POST[par];
          d.src0 = im.U[par];
          d.max0 = b.dry ? nullptr : pl.pmax + ib + par;
        }
      } else {
        if (par == s.root) {
          d.in = im.FR[s.rslot[c]];
          d.in_max = b.dry ? nullptr : pl.frmax + ib + s.rslot[c];
        } else {
          d.in = im.TMP[par];
          d.in_max = b.dry ? nullptr : pl.tmax + ib + par;
        }
        d.mode = EPI_DOWN;
        d.dst0 = im.MARG[c];
        d.src0 = im.POST[c];
        d.amax0 = b.dry ? nullptr : pl.amax + ib + c;
        if (!s.ch[c].empty()) {
          d.dst1 = im.TMP[c];
          d.src1 = im.U[c];
          d.max1 = b.dry ? nullptr : pl.tmax + ib + c;
        }
      }
      // in_M in schedule order: joint index (upward), P-1 + joint index (downward)
      d.in_max_f64 = b.dry ? nullptr
                           : pl.msgmax + (size_t)mm.img * 2 * (P - 1) + (mm.up ? 0 : P - 1) + mm.joint;
    }
    // TMA maps of what the column pass stages (plain messages only): the e2
    // buffer and the epilogue's inputs src0 / src1, [3][n] maps.  The blob
    // space is reserved alike in both passes; a map that cannot be made (a
    // caller's unaligned buffer) sends the phase to the gathering kernel.
    std::vector<CUtensorMap> maps(3 * ph.size());
    const size_t n = ph.size();
    const bool reserve = out.n_full == 0 && out.tc.empty() && !ph.empty() && W % 4 == 0;
    bool tma = reserve && !b.dry;
    for (size_t k = 0; k < n && tma; ++k) {
      const MsgDesc &d = descs[k];
      tma = make_e2_map(&maps[k], d.e2, R, H, W) &&
            (!d.src0 || make_src_map(&maps[n + k], d.src0, R, H, W)) &&
            (!d.src1 || make_src_map(&maps[2 * n + k], d.src1, R, H, W));
    }
    const CUtensorMap *tm = reserve ? b.param(maps.data(), maps.size()) : nullptr;
    out.tma = tma;
    for (size_t k = 0; k < n; ++k) {
      descs[k].tm_e2 = tma ? tm + k : nullptr;
      descs[k].tm_src0 = tma && descs[k].src0 ? tm + n + k : nullptr;
      descs[k].tm_src1 = tma && descs[k].src1 ? tm + 2 * n + k : nullptr;
    }
    out.msgs = b.param(descs.data(), descs.size());
  };
  // tables first so descriptors can point into them
  pl.tables = b.scratch<int16_t>((size_t)pl.n_msgs_total * tbl_per);
  pl.sdesc = b.scratch<int4>((size_t)pl.n_msgs_total * 4 * R);
  pl.up.assign(upph.size(), {});
  pl.down.assign(dnph.size(), {});
  for (size_t k = 0; k < upph.size(); ++k) build_phase(upph[k], upmp[k], pl.up[k]);
  for (size_t k = 0; k < dnph.size(); ++k) build_phase(dnph[k], dnmp[k], pl.down[k]);
  pl.shifts = b.param(all_shifts.data(), all_shifts.size());

  std::vector<RootDesc> rds(B);
  for (int i = 0; i < B; ++i) {
    RootDesc &rd = rds[i];
    std::memset(&rd, 0, sizeof rd);
    ImgMaps &im = pl.im[i];
    rd.k = (int)s.ch[s.root].size();
    for (int k = 0; k < rd.k; ++k) {
      rd.msg[k] = im.MSGR[k];
      rd.from_root[k] = im.FR[k];
      rd.fr_max[k] = b.dry ? nullptr : pl.frmax + i * P + k;
    }
    rd.unary = im.U[s.root];
    rd.post = im.MARG[s.root];
    rd.amax = b.dry ? nullptr : pl.amax + i * P + s.root;
  }
  pl.roots = b.param(rds.data(), rds.size());

  std::vector<int> keep;
  if (s.upright[s.root]) {  // objectdetect_findrot.cpp:698-707
    int k1 = index_from_rot(e, -1e-6), k2 = index_from_rot(e, 1e-6);
    keep.push_back(k1);
    if (k2 != k1) keep.push_back(k2);
  } else {
    for (int r = 0; r < R; ++r) keep.push_back(r);
  }
  pl.n_keep = (int)keep.size();
  pl.keep = b.param(keep.data(), keep.size());
  std::vector<const float *> pr(B);
  std::vector<float *> rp(B);
  for (int i = 0; i < B; ++i) {
    pr[i] = pl.im[i].MARG[s.root];
    rp[i] = pl.im[i].root_post;
  }
  pl.post_root_ptrs = b.param(pr.data(), pr.size());
  pl.root_post_ptrs = b.param(rp.data(), rp.size());
}

void plan_marg_ptrs(Builder &b, PsPlan &pl) {
  std::vector<const float *> mp;
  for (int i = 0; i < pl.B; ++i)
    for (int p = 0; p < pl.P; ++p) mp.push_back(pl.im[i].MARG[p]);
  pl.marg_ptrs = b.param(mp.data(), mp.size());
}

// Local maxima are computed only when some output asks for them.
void plan_localmax(Builder &b, PsPlan &pl, const pa_exp_param *e, const pa_ps_outputs *outs) {
  pl.want_part_hyps = pl.want_root_hyps = false;
  for (int i = 0; i < pl.B; ++i) {
    if (outs[i].part_hyps || outs[i].n_part_hyps) pl.want_part_hyps = true;
    if (outs[i].root_hyps || outs[i].n_root_hyps) pl.want_root_hyps = true;
  }
  pl.hyp_k = e->roi_save_num_samples;
  if (pl.hyp_k < 1) pl.want_part_hyps = false;
  if (!e->use_pairwise) pl.want_root_hyps = false;
  size_t sb = 0;
  const int hyp_maps = (pl.hyp_img >= 0 ? 1 : pl.B) * pl.P;
  const int root_maps = pl.root_joint ? 1 : pl.B;
  const int64_t root_cells = (int64_t)(pl.root_joint ? pl.B : 1) * pl.H * pl.W;
  if (pl.want_part_hyps) {
    sb = std::max(sb, local_max_scratch_bytes(hyp_maps, pl.N, pl.hyp_k));
    pl.part_hyps = b.scratch<float>((size_t)hyp_maps * pl.hyp_k * 4);
    pl.n_part_hyps = b.scratch<int>((size_t)hyp_maps);
  }
  if (pl.want_root_hyps) {
    sb = std::max(sb, local_max_scratch_bytes(root_maps, root_cells, kRootHyps));
    pl.root_hyps = b.scratch<float>((size_t)root_maps * kRootHyps * 4);
    pl.n_root_hyps = b.scratch<int>((size_t)root_maps);
  }
  pl.lm_scratch = sb ? (void *)b.scratch<char>(sb) : nullptr;
}

pa_status run_ps_tail(pa_ctx *ctx, const pa_exp_param *e, PsPlan &pl);

pa_status run_ps(pa_ctx *ctx, const pa_exp_param *e, PsPlan &pl) {
  cudaStream_t st = ctx->stream;
  const int B = pl.B, P = pl.P, R = pl.R, H = pl.H, W = pl.W;
  auto run_phase = [&](const PsPlan::Phase &ph) -> pa_status {
    PA_LAUNCH("msg_rows", launch_msg_rows(ph.msgs, ph.n, R, H, W, ph.padx, pl.err, st));
    if (ph.n_full + (int)ph.tc.size() < ph.n)
      PA_LAUNCH("msg_cols", launch_msg_cols(ph.msgs, ph.n, R, H, W, ph.pady, pl.err, st, ph.tma));
    if (ph.n_full)
      PA_LAUNCH_N("msg_full", 7, launch_msg_full(ph.msgs, ph.n, R, H, W, ph.ohmax, ph.owmax,
                                                 ph.kxf, ph.kyf, pl.err, st));
    if (!ph.tc.empty()) {
      PA_LAUNCH("msg_tc", launch_tc_toeplitz(ph.msgs, ph.n, H, W, st));
      for (const auto &j : ph.tc) {
        GemmArgs gx{};  // X^T [W][R*H] = Tx * E'^T, banded by kx, bf16 out
        gx.C = j.xt;
        gx.M = W;
        gx.N = R * H;
        gx.K = W;
        gx.ldc = (int64_t)R * H;
        gx.band = j.kx;
        gx.out_bf16 = 1;
        PA_LAUNCH("msg_tc", launch_tc_gemm(j.tbx, pl.wp, W, W, j.eb, pl.wp, (int64_t)R * H, W, gx,
                                           1, pl.err, st));
        GemmArgs gy{};  // Y_r [H][W] = Ty * X_r, banded by ky, fp32 out, batched over r
        gy.C = j.yv;
        gy.M = H;
        gy.N = W;
        gy.K = H;
        gy.ldc = W;
        gy.c_batch = (int64_t)H * W;
        gy.b_kofs = H;
        gy.band = j.ky;
        PA_LAUNCH("msg_tc", launch_tc_gemm(j.tby, pl.hp, H, H, j.xt, (int64_t)R * H, W,
                                           (int64_t)R * H, gy, R, pl.err, st));
      }
      PA_LAUNCH("msg_tc", launch_tc_epi(ph.msgs, ph.n, R, H, W, st));
    }
    return PA_OK;
  };
  if (e->use_pairwise) {
    if (pl.n_msgs_total > 0)
      PA_LAUNCH_N("shift_tables", 2, launch_shift_tables(pl.shifts, pl.n_msgs_total, R, H, W, pl.tables, pl.sdesc, st));
    for (auto &ph : pl.up) {
      if (!ph.n) continue;
      if (pa_status s2 = run_phase(ph)) return s2;
    }
    PA_LAUNCH("root_combine", launch_root_combine(pl.roots, B, pl.N,
                                                  (int)pl.sc.ch[pl.sc.root].size(), st));
    for (auto &ph : pl.down) {
      if (!ph.n) continue;
      if (pa_status s2 = run_phase(ph)) return s2;
    }
  }
  return run_ps_tail(ctx, e, pl);
}

// The PS after the messages: root rotation marginalisation (or the argmax of
// the unaries without pairwise terms), log-partition, local maxima.
pa_status run_ps_tail(pa_ctx *ctx, const pa_exp_param *e, PsPlan &pl) {
  cudaStream_t st = ctx->stream;
  const int B = pl.B, P = pl.P, R = pl.R, H = pl.H, W = pl.W;
  if (e->use_pairwise) {
    PA_LAUNCH("root_posterior", launch_root_posterior(pl.post_root_ptrs, pl.root_post_ptrs, pl.keep, pl.n_keep, B,
                                    R, H, W, st));
    // leaves without a downward message (a root without children) keep the
    // upward belief; their argmax comes from the combine kernel (root) only.
  } else {
    PA_LAUNCH("argmax", launch_argmax(pl.marg_ptrs, B * P, pl.N, pl.amax, st));
  }
  PA_LAUNCH_N("log_z", 3, launch_log_z(pl.marg_ptrs, pl.amax, B * P, pl.N, pl.logz_part, pl.logz, st));
  if (pl.want_part_hyps) {
    const int first = pl.hyp_img >= 0 ? pl.hyp_img * P : 0;
    const int n_maps = pl.hyp_img >= 0 ? P : B * P;
    static const char *names[3] = {"lm_cand", "lm_select", "lm_final"};
    for (int g = 0; g < 3; ++g)
      PA_LAUNCH_N(names[g], local_max_kernels(pl.N, pl.hyp_k, 1 << g),
                  launch_local_max(pl.marg_ptrs + first, n_maps, R, H, W, pl.hyp_k, pl.lm_scratch,
                                   pl.part_hyps, pl.n_part_hyps, st, nullptr, 1 << g));
  }
  if (pl.want_root_hyps) {
    // one [S][H][W] grid with scale neighbours (objectdetect_aux.cpp:193-236) when
    // the entries are the scales of one image, else one [1][H][W] grid per image
    const int n_maps = pl.root_joint ? 1 : B, S = pl.root_joint ? B : 1;
    static const char *names[3] = {"lm_cand", "lm_select", "lm_final"};
    for (int g = 0; g < 3; ++g)
      PA_LAUNCH_N(names[g], local_max_kernels((int64_t)S * H * W, kRootHyps, 1 << g),
                  launch_local_max(reinterpret_cast<const float *const *>(pl.root_post_ptrs),
                                   n_maps, S, H, W, kRootHyps, pl.lm_scratch, pl.root_hyps,
                                   pl.n_root_hyps, st, nullptr, 1 << g));
  }
  return PA_OK;
}

pa_status init_slots(pa_ctx *ctx, PsPlan &pl) {
  cudaStream_t st = ctx->stream;
  const int n = pl.B * pl.P;
  PA_LAUNCH("fill", launch_fill_int(pl.umax, kFkeyNegInf, n, st));
  PA_LAUNCH("fill", launch_fill_int(pl.pmax, kFkeyNegInf, n, st));
  PA_LAUNCH("fill", launch_fill_int(pl.frmax, kFkeyNegInf, n, st));
  PA_LAUNCH("fill", launch_fill_int(pl.tmax, kFkeyNegInf, n, st));
  PA_CK(cudaMemsetAsync(pl.amax, 0, sizeof(unsigned long long) * n, st));
  PA_CK(cudaMemsetAsync(pl.err, 0, sizeof(int), st));
  return PA_OK;
}

void decode_hyp(const pa_exp_param *e, unsigned long long key, int H, int W, pa_part_hyp *h,
                int scaleidx) {
  const float v = ukey_decode((uint32_t)(key >> 32));
  const uint32_t flat = 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFu);
  const int64_t HW = (int64_t)H * W;
  const int r = (int)(flat / HW);
  const int64_t rem = flat % HW;
  h->scaleidx = (float)scaleidx;
  h->scale = (float)scale_from_index(e, scaleidx);
  h->rotidx = (float)r;
  h->rot = (float)rot_from_index(e, r);
  h->x = (float)(rem % W);
  h->y = (float)(rem / W);
  h->score = v;
}

// Host landing place of the small per-call results (inside a pinned block).
struct Readback {
  unsigned long long *am = nullptr;
  double *lz = nullptr, *mm = nullptr;
  int *err = nullptr, *nph = nullptr, *nrh = nullptr;
  float *ph = nullptr, *rh = nullptr;
};

// Queues the device->host copies of a finished plan's results: the small
// ones into landing block `slot`, the maps into the caller's host outputs.
pa_status finish_enqueue(pa_ctx *ctx, const pa_exp_param *e, const PsPlan &pl,
                         const pa_ps_outputs *outs, int mem, int slot, Readback &rb) {
  const int B = pl.B, P = pl.P, H = pl.H, W = pl.W;
  const int hyp_maps = (pl.hyp_img >= 0 ? 1 : B) * P;
  const int root_maps = pl.root_joint ? 1 : B;
  const size_t n_am = (size_t)B * P, n_mm = (size_t)B * 2 * std::max(1, P - 1);
  const size_t n_ph = pl.want_part_hyps ? (size_t)hyp_maps * pl.hyp_k * 4 : 0;
  const size_t n_rh = pl.want_root_hyps ? (size_t)root_maps * kRootHyps * 4 : 0;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 15) / 16 * 16;
    return o;
  };
  const size_t o_am = carve(n_am * 8), o_lz = carve(n_am * 8), o_mm = carve(n_mm * 8),
               o_err = carve(4), o_nph = carve((size_t)hyp_maps * 4), o_nrh = carve((size_t)root_maps * 4),
               o_ph = carve(n_ph * 4), o_rh = carve(n_rh * 4);
  pa_ctx::Landing &ld = ctx->land[slot];
  if (ld.cap < off) {  // the slot's previous results were consumed before this call
    if (ld.p) cudaFreeHost(ld.p);
    ld.p = nullptr;
    ld.cap = 0;
    if (cudaMallocHost(&ld.p, off) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes of pinned result staging", off);
    }
    ld.cap = off;
  }
  rb.am = reinterpret_cast<unsigned long long *>(ld.p + o_am);
  rb.lz = reinterpret_cast<double *>(ld.p + o_lz);
  rb.mm = reinterpret_cast<double *>(ld.p + o_mm);
  rb.err = reinterpret_cast<int *>(ld.p + o_err);
  rb.nph = reinterpret_cast<int *>(ld.p + o_nph);
  rb.nrh = reinterpret_cast<int *>(ld.p + o_nrh);
  rb.ph = reinterpret_cast<float *>(ld.p + o_ph);
  rb.rh = reinterpret_cast<float *>(ld.p + o_rh);
  cudaStream_t st = ctx->stream;
  PA_CK(cudaMemcpyAsync(rb.am, pl.amax, n_am * 8, cudaMemcpyDeviceToHost, st));
  PA_CK(cudaMemcpyAsync(rb.lz, pl.logz, n_am * 8, cudaMemcpyDeviceToHost, st));
  PA_CK(cudaMemcpyAsync(rb.mm, pl.msgmax, n_mm * 8, cudaMemcpyDeviceToHost, st));
  PA_CK(cudaMemcpyAsync(rb.err, pl.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (pl.want_part_hyps) {
    PA_CK(cudaMemcpyAsync(rb.ph, pl.part_hyps, n_ph * 4, cudaMemcpyDeviceToHost, st));
    PA_CK(cudaMemcpyAsync(rb.nph, pl.n_part_hyps, (size_t)hyp_maps * 4, cudaMemcpyDeviceToHost, st));
  }
  if (pl.want_root_hyps) {
    PA_CK(cudaMemcpyAsync(rb.rh, pl.root_hyps, n_rh * 4, cudaMemcpyDeviceToHost, st));
    PA_CK(cudaMemcpyAsync(rb.nrh, pl.n_root_hyps, (size_t)root_maps * 4, cudaMemcpyDeviceToHost, st));
  }
  if (mem == PA_MEM_HOST)
    for (int i = 0; i < B; ++i) {
      const pa_ps_outputs &o = outs[i];
      if (o.log_marg)
        for (int p = 0; p < P; ++p)
          PA_CK(cudaMemcpyAsync(o.log_marg + (int64_t)p * (pl.out_pstride ? pl.out_pstride : pl.N),
                                pl.im[i].MARG[p], pl.N * sizeof(float), cudaMemcpyDeviceToHost, st));
      if (o.root_post && e->use_pairwise)
        PA_CK(cudaMemcpyAsync(o.root_post, pl.im[i].root_post, (size_t)H * W * sizeof(float),
                              cudaMemcpyDeviceToHost, st));
    }
  return PA_OK;
}

// Decodes the landed results into the host outputs (after the stream has
// passed the copies that finish_enqueue queued).
pa_status finish_complete(pa_ctx *ctx, const pa_exp_param *e, const PsPlan &pl,
                          const pa_ps_outputs *outs, const Readback &rb) {
  const int B = pl.B, P = pl.P, H = pl.H, W = pl.W;
  const int errflag = *rb.err;
  for (int i = 0; i < B; ++i) {
    const pa_ps_outputs &o = outs[i];
    const int scaleidx = pl.img_scale.empty() ? 0 : pl.img_scale[i];
    // this entry's row in the local-maximum results (-1: none computed)
    const int hrow = pl.hyp_img < 0 ? i : (pl.hyp_img == i ? 0 : -1);
    for (int p = 0; p < P; ++p) {
      if (o.best) decode_hyp(e, rb.am[(size_t)i * P + p], H, W, &o.best[p], scaleidx);
      if (o.log_z) o.log_z[p] = rb.lz[(size_t)i * P + p];
      const int n = pl.want_part_hyps && hrow >= 0 ? rb.nph[(size_t)hrow * P + p] : 0;
      if (o.n_part_hyps) o.n_part_hyps[p] = n;
      if (o.part_hyps)
        for (int k = 0; k < n; ++k) {
          // PartHyp(exp_param, 0, rotidx, x, y, score).toVect(), objectdetect.h:95-159
          const float *r = &rb.ph[(((size_t)hrow * P + p) * pl.hyp_k + k) * 4];
          pa_part_hyp &h = o.part_hyps[(size_t)p * pl.hyp_k + k];
          h.scaleidx = 0.f;
          h.scale = (float)scale_from_index(e, 0);
          h.rotidx = r[0];
          h.rot = (float)rot_from_index(e, (int)r[0]);
          h.x = r[1];
          h.y = r[2];
          h.score = r[3];
        }
    }
    if (o.msg_max)
      for (int k = 0; k < 2 * (P - 1); ++k) o.msg_max[k] = rb.mm[(size_t)i * 2 * (P - 1) + k];
    const int rrow = pl.root_joint ? (i == 0 ? 0 : -1) : i;
    const int nr = pl.want_root_hyps && rrow >= 0 ? rb.nrh[rrow] : 0;
    if (o.n_root_hyps) *o.n_root_hyps = nr;
    if (o.root_hyps)
      for (int k = 0; k < nr; ++k) {
        // ObjectHypothesis (scale, x, y, score), objectdetect_aux.cpp:279-290
        const float *r = &rb.rh[((size_t)rrow * kRootHyps + k) * 4];
        o.root_hyps[4 * k + 0] = (float)scale_from_index(e, (int)r[0]);
        o.root_hyps[4 * k + 1] = r[1];
        o.root_hyps[4 * k + 2] = r[2];
        o.root_hyps[4 * k + 3] = r[3];
      }
  }
  if (errflag & 1)
    return fail(ctx, PA_ERR_NUMERIC, "exp() overflowed in a message (the reference asserts here)");
  if (errflag & 8)
    return fail(ctx, PA_ERR_CUDA, "tensor-core pipeline wait timed out (code %d)", errflag);
  if (errflag & ~1)
    return fail(ctx, PA_ERR_UNSUPPORTED, "message kernel rejected its input (code %d)", errflag);
  return PA_OK;
}

// Reads back the small per-image results and writes host outputs.
pa_status finish_ps(pa_ctx *ctx, const pa_exp_param *e, PsPlan &pl, const pa_ps_outputs *outs,
                    int mem) {
  Readback rb;
  if (pa_status st = finish_enqueue(ctx, e, pl, outs, mem, 0, rb)) return st;
  if (pa_status st = sync_ctx(ctx)) return st;
  return finish_complete(ctx, e, pl, outs, rb);
}

// Unary-map descriptors for B images x P parts x R rotations.
struct UnaryTables {
  std::vector<int> colx, rowy;
  std::vector<float> cola, rowb;
  bool separable = false;
  bool collide = false;  // TM_DIRECT: two grid cells may round to one pixel
  double T13[9], T31[9];
};

// plan_unary's flags: every map takes the separable bilinear kernel; some
// direct map keeps a last-writer scratch (a third launch)
constexpr int kUnarySeparable = 1, kUnaryOrdered = 2;
int unary_launches(int direct, int flags) {
  return !direct ? 1 : (flags & kUnaryOrdered) ? 3 : 2;
}

pa_status unary_tables(pa_ctx *ctx, const double *Tig, int ny, int nx, int H, int W, int direct,
                       UnaryTables &t) {
  for (int k = 0; k < 9; ++k) t.T31[k] = Tig[k];
  if (Tig[6] != 0 || Tig[7] != 0 || Tig[8] != 1)
    return fail(ctx, PA_ERR_INVALID, "Tig must be affine (last row 0 0 1)");
  hc_inverse(Tig, t.T13);
  if (!std::isfinite(t.T13[0]) || !std::isfinite(t.T13[4]))
    return fail(ctx, PA_ERR_INVALID, "Tig is singular");
  if (!direct) {
    t.separable = (t.T13[1] == 0 && t.T13[3] == 0);
    if (t.separable) {
      t.colx.resize(W);
      t.cola.resize(W);
      t.rowy.resize(H);
      t.rowb.resize(H);
      for (int x3 = 0; x3 < W; ++x3) {
        double x1 = t.T13[0] * x3 + t.T13[2];
        int ix = (int)std::floor(x1);
        t.colx[x3] = ix;
        t.cola[x3] = (float)(x1 - ix);
      }
      for (int y3 = 0; y3 < H; ++y3) {
        double y1 = t.T13[4] * y3 + t.T13[5];
        int iy = (int)std::floor(y1);
        t.rowy[y3] = iy;
        t.rowb[y3] = (float)(y1 - iy);
      }
    }
  } else {
    t.separable = (Tig[1] == 0 && Tig[3] == 0);
    if (t.separable) {
      t.colx.resize(nx);
      t.rowy.resize(ny);
      for (int x1 = 0; x1 < nx; ++x1) t.colx[x1] = (int)std::floor(Tig[0] * x1 + Tig[2] + 0.5);
      for (int y1 = 0; y1 < ny; ++y1) t.rowy[y1] = (int)std::floor(Tig[4] * y1 + Tig[5] + 0.5);
      std::vector<int> cx(t.colx), ry(t.rowy);
      std::sort(cx.begin(), cx.end());
      std::sort(ry.begin(), ry.end());
      t.collide = std::adjacent_find(cx.begin(), cx.end()) != cx.end() ||
                  std::adjacent_find(ry.begin(), ry.end()) != ry.end();
    } else {
      // cells one grid step apart land more than sqrt 2 apart, so never on one
      // pixel, when the smallest singular value of the linear part exceeds sqrt 2
      const double a = Tig[0], b = Tig[1], c = Tig[3], d = Tig[4];
      const double s1 = a * a + b * b + c * c + d * d, det = std::fabs(a * d - b * c);
      const double smin2 = 0.5 * (s1 - std::sqrt(std::max(0.0, s1 * s1 - 4 * det * det)));
      t.collide = !(smin2 > 2.0);
    }
  }
  return PA_OK;
}

pa_status plan_unary(pa_ctx *ctx, Builder &b, const double *Tig, int tig_shared, int n_img, int P,
                     int R, int ny, int nx, int H, int W, int direct, const float *scores,
                     int64_t scores_field_stride, const std::vector<std::vector<float *>> &outs,
                     const std::vector<int> &upright, int root, float strip_frac, int *umax,
                     const pa_exp_param *e, UnaryMap **maps_dev, int apply_masks,
                     int *flags) {
  const int n_tig = tig_shared ? 1 : P * R;
  std::vector<UnaryTables> tabs(n_tig);
  std::vector<const int *> dcolx(n_tig), drowy(n_tig);
  std::vector<const float *> dcola(n_tig), drowb(n_tig);
  for (int k = 0; k < n_tig; ++k) {
    pa_status st = unary_tables(ctx, Tig + 9 * k, ny, nx, H, W, direct, tabs[k]);
    if (st) return st;
    if (tabs[k].separable) {
      dcolx[k] = b.param(tabs[k].colx.data(), tabs[k].colx.size());
      drowy[k] = b.param(tabs[k].rowy.data(), tabs[k].rowy.size());
      if (!direct) {
        dcola[k] = b.param(tabs[k].cola.data(), tabs[k].cola.size());
        drowb[k] = b.param(tabs[k].rowb.data(), tabs[k].rowb.size());
      }
    }
  }
  const int strip = (int)(strip_frac * W);
  *flags = kUnarySeparable;
  bool any_collide = false;
  for (int k = 0; k < n_tig; ++k) {
    if (!tabs[k].separable || std::fabs(tabs[k].T13[4]) > 1.0) *flags = 0;
    any_collide = any_collide || (direct && tabs[k].collide);
  }
  // last-writer scratch for the maps whose cells may share a pixel
  int *order = any_collide ? b.scratch<int>((size_t)n_img * P * R * H * W) : nullptr;
  if (any_collide) *flags |= kUnaryOrdered;
  std::vector<UnaryMap> maps((size_t)n_img * P * R);
  for (int i = 0; i < n_img; ++i)
    for (int p = 0; p < P; ++p)
      for (int r = 0; r < R; ++r) {
        UnaryMap &m = maps[((size_t)i * P + p) * R + r];
        std::memset(&m, 0, sizeof m);
        const int k = tig_shared ? 0 : p * R + r;
        m.grid = b.dry ? nullptr : scores + ((int64_t)p * scores_field_stride + (int64_t)i * R + r) * ny * nx;
        m.out = b.dry ? nullptr : outs[i][p] + (int64_t)r * H * W;
        m.separable = tabs[k].separable;
        m.colx = dcolx[k];
        m.cola = dcola[k];
        m.rowy = drowy[k];
        m.rowb = drowb[k];
        for (int q = 0; q < 6; ++q) {
          m.T13[q] = tabs[k].T13[q];
          m.T31[q] = tabs[k].T31[q];
        }
        if (apply_masks) {
          m.masked_all = upright[p] && !(std::fabs(rot_from_index(e, r)) < 15.0);
          m.strip = (p == root) ? strip : 0;
        }
        m.max_slot = (b.dry || !umax) ? nullptr : umax + i * P + p;
        m.order = (order && tabs[k].collide) ? order + (((size_t)i * P + p) * R + r) * H * W
                                             : nullptr;
      }
  *maps_dev = b.param(maps.data(), maps.size());
  return PA_OK;
}

pa_status check_classifiers(pa_ctx *ctx, const pa_classifier *const *cls, int n_parts, int dim) {
  if (!cls || n_parts < 1) return fail(ctx, PA_ERR_INVALID, "no classifiers");
  for (int p = 0; p < n_parts; ++p) {
    if (!cls[p]) return fail(ctx, PA_ERR_INVALID, "classifier %d is NULL", p);
    if (cls[p]->dim != dim)
      return fail(ctx, PA_ERR_INVALID, "classifier %d has dim %d, descriptors have %d", p,
                  cls[p]->dim, dim);
  }
  return PA_OK;
}

// Rank tables of a classifier set (the rank form of k_stump.cu), built once
// per set and context.  nullptr when the set does not qualify: a polarity
// other than +-1, more than 127 distinct thresholds on one feature, dim >
// 1023 or not a multiple of 4, more than 32 classifiers, or tables beyond
// shared memory.
const RankTables *rank_tables(pa_ctx *ctx, const pa_classifier *const *cls, int n) {
  std::vector<uint64_t> key(n);
  for (int c = 0; c < n; ++c) key[c] = cls[c]->id;
  auto it = ctx->rank_sets.find(key);
  if (it != ctx->rank_sets.end()) return it->second.ok ? &it->second.rt : nullptr;
  pa_ctx::RankEntry &ent = ctx->rank_sets[key];
  const int dim = cls[0]->dim;
  if (n < 1 || n > 32 || dim > 1023 || dim % 4) return nullptr;
  int nmax = 0;
  for (int c = 0; c < n; ++c) {
    if (cls[c]->dim != dim || cls[c]->fast_h.empty()) return nullptr;
    nmax = std::max(nmax, cls[c]->n);
  }
  const int npad = (nmax + 3) / 4 * 4;
  if (rank_votes_smem(dim, n, npad) > 227 * 1024) return nullptr;
  // distinct thresholds per feature, ascending (-0 and +0 are one value)
  std::vector<std::vector<float>> U(dim);
  for (int c = 0; c < n; ++c)
    for (const float4 &q : cls[c]->fast_h) {
      int f;
      std::memcpy(&f, &q.x, 4);
      U[f].push_back(q.y);
    }
  size_t mmax = 0;
  for (auto &u : U) {
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end(), [](float a, float b) { return a == b; }), u.end());
    mmax = std::max(mmax, u.size());
  }
  if (mmax > 127) return nullptr;
  int d = 1;
  while (((size_t)1 << d) - 1 < mmax) ++d;
  const int S = (1 << d) + 1, top = 1 << d;
  // Eytzinger order: e[1] the root, children of e[i] at 2i and 2i + 1 (an
  // in-order walk of that tree visits the sorted thresholds, +inf padded)
  std::vector<float> eyt((size_t)dim * S, INFINITY);
  for (int f = 0; f < dim; ++f) {
    size_t next = 0;
    float *row = eyt.data() + (size_t)f * S;
    std::function<void(int)> fill = [&](int i) {
      if (i >= top) return;
      fill(2 * i);
      row[i] = next < U[f].size() ? U[f][next] : INFINITY;
      ++next;
      fill(2 * i + 1);
    };
    fill(1);
  }
  std::vector<uint2> rec((size_t)n * npad, make_uint2(0xFFu << 24, 0x80000000u));
  std::vector<float> sa(n);
  for (int c = 0; c < n; ++c) {
    sa[c] = cls[c]->sum_alpha;
    for (int i = 0; i < cls[c]->n; ++i) {
      const float4 &q = cls[c]->fast_h[i];
      int f;
      std::memcpy(&f, &q.x, 4);
      const auto &u = U[f];
      const uint32_t k = (uint32_t)(std::lower_bound(u.begin(), u.end(), q.y) - u.begin());
      const float na = -q.z;
      uint32_t nab;
      std::memcpy(&nab, &na, 4);
      rec[(size_t)c * npad + i] = make_uint2((uint32_t)f * 128u | ((0x80u + k) << 24), nab);
    }
  }
  const size_t b_eyt = eyt.size() * sizeof(float), b_rec = rec.size() * sizeof(uint2);
  const size_t o_rec = (b_eyt + 255) / 256 * 256, o_sa = o_rec + (b_rec + 255) / 256 * 256;
  char *mem = nullptr;
  if (cudaMalloc(&mem, o_sa + sa.size() * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (cudaMemcpy(mem, eyt.data(), b_eyt, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(mem + o_rec, rec.data(), b_rec, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(mem + o_sa, sa.data(), sa.size() * sizeof(float), cudaMemcpyHostToDevice) !=
          cudaSuccess) {
    cudaGetLastError();
    cudaFree(mem);
    return nullptr;
  }
  ent.mem = mem;
  ent.rt.eyt = reinterpret_cast<const float *>(mem);
  ent.rt.rec = reinterpret_cast<const uint2 *>(mem + o_rec);
  ent.rt.sum_alpha = reinterpret_cast<const float *>(mem + o_sa);
  ent.rt.d = d;
  ent.rt.dim = dim;
  ent.rt.n_cls = n;
  ent.rt.npad = npad;
  ent.ok = true;
  return &ent.rt;
}

StumpPart *plan_stumps(Builder &b, const pa_classifier *const *cls, int n_parts) {
  std::vector<StumpPart> sp(n_parts);
  for (int p = 0; p < n_parts; ++p) {
    const pa_classifier *c = cls[p];
    sp[p].stumps = c->d;
    sp[p].fast = c->fast;
    sp[p].f8 = c->packed ? reinterpret_cast<const uint4 *>(c->packed) : nullptr;
    sp[p].ta2 = c->packed ? reinterpret_cast<const float4 *>(c->packed + (size_t)c->npad * 2) : nullptr;
    sp[p].n = c->n;
    sp[p].npad = c->npad;
    sp[p].sum_alpha = c->sum_alpha;
  }
  return b.param(sp.data(), sp.size());
}

std::vector<char> fast_flags(const pa_classifier *const *cls, int n) {
  std::vector<char> f(n);
  for (int p = 0; p < n; ++p) f[p] = cls[p]->packed != nullptr;
  return f;
}

std::vector<int> stump_counts(const pa_classifier *const *cls, int n) {
  std::vector<int> c(n);
  for (int p = 0; p < n; ++p) c[p] = cls[p]->npad ? cls[p]->npad : cls[p]->n;
  return c;
}

// The whole --find_obj pipeline for n_img images.
// scores_out (if any) is laid out [n_cls][scores_fields][ny][nx] and this
// call fills fields [scores_field0, scores_field0 + n_img*R) of it.
// An image whose results are still on their way to the host: its plan, the
// landing slot of its small results and its outputs.
}  // namespace

// ------------------------------------------------------------------------
// Learned unary (no reference counterpart): network state and the layer
// sequence of its forward and backward passes.
// ------------------------------------------------------------------------
struct pa_unary_net {
  int device = 0;
  int dim = 0, P = 0;
  int64_t off_w[5] = {}, off_b[5] = {}, n_params = 0;
  float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  __nv_bfloat16 *wf0 = nullptr, *wf[4] = {}, *wd[4] = {};
  int64_t step = 0;  // Adam steps taken
  char *scratch = nullptr;
  size_t scratch_cap = 0;
  int *err = nullptr;
};

namespace {

void net_layout(pa_unary_net *n) {
  int64_t o = 0;
  for (int l = 0; l < 5; ++l) {
    const int64_t cout = l == 4 ? n->P : 64, k = l == 0 ? n->dim : 576;
    n->off_w[l] = o;
    o += cout * k;
    n->off_b[l] = o;
    o += cout;
  }
  n->n_params = o;
}

struct NetScratch {
  __nv_bfloat16 *x = nullptr;       // BF16 copy of FP32 fields
  __nv_bfloat16 *act[4] = {};       // post-ReLU activations of layers 0..3
  float *y = nullptr;               // training: output log scores [P][n][ny][nx]
  __nv_bfloat16 *dz4 = nullptr, *dza = nullptr, *dzb = nullptr;
  float *wpart = nullptr;
  size_t wpart_floats = 0;
  float *bpart = nullptr;
  float *lpart = nullptr;
  double *loss = nullptr;
};
constexpr int kBiasBlocks = 256;

pa_status net_scratch(pa_ctx *ctx, pa_unary_net *net, int n, int ny, int nx, bool cast,
                      bool train, NetScratch &sc) {
  const size_t L = (size_t)n * ny * nx;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = (off + 255) / 256 * 256;
    off = o + bytes;
    return o;
  };
  const size_t ox = cast ? take(L * net->dim * 2) : 0;
  size_t oa[4];
  for (int l = 0; l < 4; ++l) oa[l] = take(L * 64 * 2);
  size_t oy = 0, od4 = 0, oda = 0, odb = 0, ow = 0, ob = 0, ol = 0, olo = 0, wf = 0;
  if (train) {
    oy = take(L * net->P * 4);
    od4 = take(L * 64 * 2);
    oda = take(L * 64 * 2);
    odb = take(L * 64 * 2);
    wf = std::max(conv_wgrad_part_floats(net->dim, 1, n, ny, nx),
                  conv_wgrad_part_floats(64, 9, n, ny, nx));
    ow = take(wf * 4);
    ob = take((size_t)kBiasBlocks * 64 * 4);
    ol = take((size_t)loss_blocks((int64_t)L) * 4);
    olo = take(8);
  }
  if (off > net->scratch_cap) {
    PA_CK(cudaStreamSynchronize(ctx->stream));
    if (net->scratch) cudaFree(net->scratch);
    net->scratch = nullptr;
    net->scratch_cap = 0;
    const size_t cap = off + off / 8 + 4096;
    if (cudaMalloc(&net->scratch, cap) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes for the unary net", cap);
    }
    net->scratch_cap = cap;
  }
  char *b = net->scratch;
  sc = NetScratch{};
  if (cast) sc.x = reinterpret_cast<__nv_bfloat16 *>(b + ox);
  for (int l = 0; l < 4; ++l) sc.act[l] = reinterpret_cast<__nv_bfloat16 *>(b + oa[l]);
  if (train) {
    sc.y = reinterpret_cast<float *>(b + oy);
    sc.dz4 = reinterpret_cast<__nv_bfloat16 *>(b + od4);
    sc.dza = reinterpret_cast<__nv_bfloat16 *>(b + oda);
    sc.dzb = reinterpret_cast<__nv_bfloat16 *>(b + odb);
    sc.wpart = reinterpret_cast<float *>(b + ow);
    sc.wpart_floats = wf;
    sc.bpart = reinterpret_cast<float *>(b + ob);
    sc.lpart = reinterpret_cast<float *>(b + ol);
    sc.loss = reinterpret_cast<double *>(b + olo);
  }
  return PA_OK;
}

pa_status net_check_fields(pa_ctx *ctx, const pa_unary_net *net, const void *fields, int n, int ny,
                           int nx) {
  if (!net || !fields || n < 1 || ny < 1 || nx < 1 || n > 65535 || ny > 65535 ||
      ((uintptr_t)fields & 15))
    return fail(ctx, PA_ERR_INVALID, "invalid net input (NULL, sizes or alignment)");
  return PA_OK;
}

pa_status net_pack(pa_ctx *ctx, pa_unary_net *net) {
  PackArgs a{};
  a.dim = net->dim;
  a.P = net->P;
  for (int l = 0; l < 5; ++l) a.off_w[l] = net->off_w[l];
  a.wf0 = net->wf0;
  for (int l = 0; l < 4; ++l) {
    a.wf[l] = net->wf[l];
    a.wd[l] = net->wd[l];
  }
  PA_LAUNCH("net_pack", launch_pack_weights(net->params, a, ctx->stream));
  return PA_OK;
}

// Forward pass, queued on the context's stream.  `out` spec as
// pa_unary_net_forward.
pa_status net_forward(pa_ctx *ctx, pa_unary_net *net, const void *fields, int bf16, int n, int ny,
                      int nx, float *out, int64_t sf, int64_t sc_, int exp_out, NetScratch &sc) {
  cudaStream_t s = ctx->stream;
  const void *x = fields;
  if (!bf16) {
    PA_LAUNCH("net_cast", launch_cast_bf16(reinterpret_cast<const float *>(fields), sc.x,
                                           (int64_t)n * ny * nx * net->dim, s));
    x = sc.x;
  }
  ConvArgs a{};
  a.mode = kConvReluBf16;
  a.bias = net->params + net->off_b[0];
  a.out = sc.act[0];
  PA_LAUNCH("net_conv", launch_conv(x, net->dim, 1, n, ny, nx, net->wf0, a, net->err, s));
  for (int l = 1; l < 4; ++l) {
    a.bias = net->params + net->off_b[l];
    a.out = sc.act[l];
    PA_LAUNCH("net_conv", launch_conv(sc.act[l - 1], 64, 9, n, ny, nx, net->wf[l - 1], a, net->err, s));
  }
  a.mode = kConvOutF32;
  a.bias = net->params + net->off_b[4];
  a.out = out;
  a.n_out = net->P;
  a.out_sf = sf;
  a.out_sc = sc_;
  a.exp_out = exp_out;
  PA_LAUNCH("net_conv", launch_conv(sc.act[3], 64, 9, n, ny, nx, net->wf[3], a, net->err, s));
  return PA_OK;
}

// Forward, loss and the gradient of every parameter (into net->grads),
// queued on the context's stream; the loss lands in *sc.loss.
pa_status net_backward(pa_ctx *ctx, pa_unary_net *net, const void *fields, int bf16,
                       const float *scores, int n, int ny, int nx, NetScratch &sc) {
  cudaStream_t s = ctx->stream;
  const int64_t G = (int64_t)ny * nx, L = (int64_t)n * G;
  if (pa_status st = net_forward(ctx, net, fields, bf16, n, ny, nx, sc.y, G, n * G, 0, sc)) return st;
  const void *x = bf16 ? fields : sc.x;
  LossArgs la{};
  la.pred = sc.y;
  la.scores = scores;
  la.pred_sf = la.score_sf = G;
  la.pred_sc = la.score_sc = n * G;
  la.n = n;
  la.P = net->P;
  la.H = ny;
  la.W = nx;
  la.inv_count = (float)(1.0 / ((double)L * net->P));
  PA_LAUNCH_N("net_loss", 2, launch_loss_grad(la, sc.dz4, sc.lpart, sc.loss, s));
  // layer l: input in[l], output gradient dz[l]; the input gradient of
  // layer l (l >= 1), masked by ReLU, is the output gradient of layer l - 1
  const void *in[5] = {x, sc.act[0], sc.act[1], sc.act[2], sc.act[3]};
  __nv_bfloat16 *dz = sc.dz4;
  for (int l = 4; l >= 0; --l) {
    const int cin = l == 0 ? net->dim : 64, taps = l == 0 ? 1 : 9, cout = l == 4 ? net->P : 64;
    PA_LAUNCH_N("net_wgrad", 2, launch_conv_wgrad(in[l], cin, taps, dz, n, ny, nx, cout, sc.wpart,
                                                  sc.wpart_floats, net->grads + net->off_w[l],
                                                  net->err, s));
    PA_LAUNCH_N("net_bgrad", 2, launch_bias_grad(dz, L, cout, sc.bpart, kBiasBlocks,
                                                 net->grads + net->off_b[l], s));
    if (l == 0) break;
    __nv_bfloat16 *next = (dz == sc.dza) ? sc.dzb : sc.dza;
    ConvArgs a{};
    a.mode = kConvMaskBf16;
    a.act = sc.act[l - 1];
    a.out = next;
    PA_LAUNCH("net_dgrad", launch_conv(dz, 64, 9, n, ny, nx, net->wd[l - 1], a, net->err, s));
    dz = next;
  }
  return PA_OK;
}

pa_status net_err_check(pa_ctx *ctx, pa_unary_net *net) {
  int flag = 0;
  PA_CK(cudaMemcpyAsync(&flag, net->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (pa_status st = sync_ctx(ctx)) return st;
  if (flag) return fail(ctx, PA_ERR_CUDA, "unary net pipeline wait timed out (flag %d)", flag);
  return PA_OK;
}

// Learned unary of find_obj_core: the net's scores for the parts on the
// net, AdaBoost for the others.
struct LearnedUnary {
  pa_unary_net *net = nullptr;
  const void *fields = nullptr;  // BF16 [n_fields][ny][nx][dim]
  std::vector<char> on_net;      // per part
  bool any_net = false, any_ada = false;
};

struct PendingImage {
  PsPlan pl;
  Readback rb;
  const pa_ps_outputs *outs = nullptr;
  int slot = 0;
  bool busy = false;
};

// `defer` null: runs the batch and returns with its results written.
// `defer` set: only queues the work and the result copies (landing slot
// defer->slot); the caller completes it with finish_complete once the
// stream has passed them.
pa_status find_obj_core(pa_ctx *ctx, const pa_exp_param *e, int n_img, const pa_tree *trees,
                        int flip, const pa_classifier *const *cls, int n_cls, const float *desc,
                        const float *const *img_desc, int in_mem, int ny, int nx, int dim,
                        const double *Tig, int tig_shared,
                        int H, int W, float *scores_out, int64_t scores_field0,
                        int64_t scores_fields, const pa_ps_outputs *outs, int mem,
                        PendingImage *defer = nullptr, const LearnedUnary *lu = nullptr) {
  PsPlan pl;
  pl.tc_mode = ctx->msg_math == PA_MSG_BF16_TENSOR;
  pl.sparse_up = true;  // findObjectImageRotJoints passes bIsSparse = true (objectdetect_findrot.cpp:740)
  pa_status st = build_sched(ctx, &trees[0], pl.sc);
  if (st) return st;
  for (int i = 1; i < n_img; ++i)
    if (!same_topology(&trees[0], &trees[i]))
      return fail(ctx, PA_ERR_INVALID, "image %d: tree topology differs from image 0", i);
  const int P = pl.sc.P, R = e->num_rotation_steps;
  // the AdaBoost classifiers are evaluated unless every part is on the net;
  // with a learned unary only those of the parts off the net, in one launch
  const bool ada = !lu || lu->any_ada;
  std::vector<const pa_classifier *> ada_cls;
  std::vector<int> ada_part;
  if (lu) {
    for (int p = 0; p < (int)lu->on_net.size() && p < n_cls; ++p)
      if (!lu->on_net[p]) {
        ada_cls.push_back(cls[p]);
        ada_part.push_back(p);
      }
  }
  const pa_classifier *const *run_cls = lu ? ada_cls.data() : cls;
  const int n_run = lu ? (int)ada_cls.size() : n_cls;
  if (lu && (int)lu->on_net.size() != P)
    return fail(ctx, PA_ERR_INVALID, "the net's part count differs from the tree's");
  if (n_cls < P) return fail(ctx, PA_ERR_INVALID, "need at least n_parts classifiers");
  if (ada && (st = check_classifiers(ctx, cls, n_cls, dim))) return st;
  std::vector<std::vector<Joint>> joints(n_img);
  for (int i = 0; i < n_img; ++i) {
    st = load_joints(ctx, &trees[i], flip, joints[i]);
    if (st) return st;
  }
  pl.B = n_img;
  pl.P = P;
  pl.R = R;
  pl.H = H;
  pl.W = W;
  pl.N = (int64_t)R * H * W;
  const int64_t G = (int64_t)ny * nx;
  const int64_t n_fields = (int64_t)n_img * R;

  std::vector<float *> marg_out(n_img, nullptr), rp_out(n_img, nullptr);
  if (mem == PA_MEM_DEVICE)
    for (int i = 0; i < n_img; ++i) {
      marg_out[i] = outs[i].log_marg;
      rp_out[i] = outs[i].root_post;
    }

  DeviceGuard dg(ctx->device);
  // pass 1 (dry): measure
  Builder b1;
  b1.dry = true;
  // device score grids can be written in place only when the caller's layout
  // is exactly this call's [n_cls][n_fields] block
  const bool scores_dev_out =
      (mem == PA_MEM_DEVICE && scores_out && scores_field0 == 0 && scores_fields == n_fields);
  StumpPart *sp = ada ? plan_stumps(b1, run_cls, n_run) : nullptr;
  // rank form of the stump test when the classifier set qualifies
  const RankTables *rk = (!lu) ? rank_tables(ctx, cls, n_cls) : nullptr;
  uint32_t *ranks = rk ? b1.scratch<uint32_t>(rank_bytes(dim, G, (int)n_fields) / 4) : nullptr;
  const float *desc_dev = (in_mem == PA_MEM_DEVICE) ? desc : b1.scratch<float>(n_fields * G * dim);
  // scores of the AdaBoost parts when the net writes the others
  const bool split_scores = lu && lu->any_ada && lu->any_net;
  float *ada_scores = split_scores ? b1.scratch<float>((size_t)n_run * n_fields * G) : nullptr;
  // per-field descriptor pointers when the images are separate device buffers
  std::vector<const float *> fptr;
  bool fields_al = true;
  if (img_desc) {
    for (int i = 0; i < n_img; ++i)
      for (int r = 0; r < R; ++r) {
        fptr.push_back(img_desc[i] + (size_t)r * G * dim);
        fields_al = fields_al && ((uintptr_t)fptr.back() & 15) == 0;
      }
  }
  const float *const *fields_dev = img_desc ? b1.param(fptr.data(), fptr.size()) : nullptr;
  float *scores = scores_dev_out ? scores_out : b1.scratch<float>((size_t)n_cls * n_fields * G);
  plan_ps(b1, pl, e, joints, marg_out.data(), rp_out.data());
  plan_marg_ptrs(b1, pl);
  plan_localmax(b1, pl, e, outs);
  UnaryMap *umaps = nullptr;
  int usep = 0;
  std::vector<std::vector<float *>> uouts(n_img, std::vector<float *>(P, nullptr));
  st = plan_unary(ctx, b1, Tig, tig_shared, n_img, P, R, ny, nx, H, W, !e->interpolate, scores,
                  n_fields, uouts, pl.sc.upright, pl.sc.root, e->strip_border_detections,
                  pl.umax, e, &umaps, 1, &usep);
  if (st) return st;
  // pass 2: real
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  st = ensure_arena(ctx, b1.total());
  if (st) return st;
  b.base = ctx->arena;
  PsPlan pl2 = pl;
  sp = ada ? plan_stumps(b, run_cls, n_run) : nullptr;
  ranks = rk ? b.scratch<uint32_t>(rank_bytes(dim, G, (int)n_fields) / 4) : nullptr;
  desc_dev = (in_mem == PA_MEM_DEVICE) ? desc : b.scratch<float>(n_fields * G * dim);
  ada_scores = split_scores ? b.scratch<float>((size_t)n_run * n_fields * G) : nullptr;
  fields_dev = img_desc ? b.param(fptr.data(), fptr.size()) : nullptr;
  scores = scores_dev_out ? scores_out : b.scratch<float>((size_t)n_cls * n_fields * G);
  plan_ps(b, pl2, e, joints, marg_out.data(), rp_out.data());
  plan_marg_ptrs(b, pl2);
  plan_localmax(b, pl2, e, outs);
  for (int i = 0; i < n_img; ++i)
    for (int p = 0; p < P; ++p) uouts[i][p] = pl2.im[i].U[p];
  st = plan_unary(ctx, b, Tig, tig_shared, n_img, P, R, ny, nx, H, W, !e->interpolate, scores,
                  n_fields, uouts, pl2.sc.upright, pl2.sc.root, e->strip_border_detections,
                  pl2.umax, e, &umaps, 1, &usep);
  if (st) return st;
  if (b.blob.size() != b1.blob.size() || b.scratch_off != b1.scratch_off)
    return fail(ctx, PA_ERR_INVALID, "internal: plan size mismatch");

  st = upload_blob(ctx, b);
  if (st) return st;
  if (in_mem == PA_MEM_HOST) {
    st = copy_in(ctx, (void *)desc_dev, desc, (size_t)n_fields * G * dim * sizeof(float), in_mem);
    if (st) return st;
  }
  st = init_slots(ctx, pl2);
  if (st) return st;
  cudaStream_t s = ctx->stream;
  if (rk) {
    const bool al = fields_dev ? fields_al : ((uintptr_t)desc_dev & 15) == 0;
    PA_LAUNCH("stump_ranks", launch_rank_buckets(*rk, desc_dev, fields_dev, al, G, (int)n_fields, ranks, s));
    PA_LAUNCH("stump_votes", launch_rank_votes(*rk, G, (int)n_fields, 1, scores, ranks, pl2.err, s));
  } else if (!lu) {
    const std::vector<char> ff = fast_flags(cls, n_cls);
    const std::vector<int> ns = stump_counts(cls, n_cls);
    PA_LAUNCH("score_grids", launch_score_grids(sp, (const bool *)ff.data(), ns.data(), n_cls, desc_dev, fields_dev, fields_al, G,
                                                (int)n_fields, dim, 1, scores, s));
  } else {
    // the net writes the scores of all P parts ([part][field][ny][nx]); the
    // AdaBoost parts are then overwritten with their classifiers' grids
    if (lu->any_net) {
      NetScratch nsc;
      if ((st = net_scratch(ctx, lu->net, (int)n_fields, ny, nx, false, false, nsc))) return st;
      PA_CK(cudaMemsetAsync(lu->net->err, 0, sizeof(int), s));
      if ((st = net_forward(ctx, lu->net, lu->fields, 1, (int)n_fields, ny, nx, scores, G,
                            n_fields * G, 1, nsc)))
        return st;
    }
    if (lu->any_ada) {
      const std::vector<char> ff = fast_flags(run_cls, n_run);
      const std::vector<int> ns = stump_counts(run_cls, n_run);
      PA_LAUNCH("score_grids", launch_score_grids(sp, (const bool *)ff.data(), ns.data(), n_run, desc_dev, nullptr,
                                                  false, G, (int)n_fields, dim, 1,
                                                  split_scores ? ada_scores : scores, s));
      if (split_scores)
        for (int k = 0; k < n_run; ++k)
          PA_CK(cudaMemcpyAsync(scores + (size_t)ada_part[k] * n_fields * G,
                                ada_scores + (size_t)k * n_fields * G,
                                (size_t)n_fields * G * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
  }
  if (scores_out && !scores_dev_out)
    PA_CK(cudaMemcpy2DAsync(scores_out + scores_field0 * G, (size_t)scores_fields * G * sizeof(float),
                            scores, (size_t)n_fields * G * sizeof(float),
                            (size_t)n_fields * G * sizeof(float), (size_t)n_cls,
                            mem == PA_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                            s));
  PA_LAUNCH_N("unary_maps", unary_launches(!e->interpolate, usep),
              launch_unary_maps(umaps, n_img * P * R, ny, nx, H, W, !e->interpolate,
                                usep & kUnarySeparable, usep & kUnaryOrdered, s));
  if (!e->use_pairwise) {
    // getMaxStates: the marginals are the masked unaries
    for (int i = 0; i < n_img; ++i)
      for (int p = 0; p < P; ++p)
        PA_CK(cudaMemcpyAsync(pl2.im[i].MARG[p], pl2.im[i].U[p], pl2.N * sizeof(float),
                              cudaMemcpyDeviceToDevice, s));
  }
  st = run_ps(ctx, e, pl2);
  if (st) return st;
  if (defer) {
    defer->pl = std::move(pl2);
    defer->outs = outs;
    return finish_enqueue(ctx, e, defer->pl, outs, mem, defer->slot, defer->rb);
  }
  return finish_ps(ctx, e, pl2, outs, mem);
}

// Host descriptors, several images: images go through a ring of device
// slots.  The copy of image i + k (k < slots) runs on the context's copy
// stream while image i is computed; the host plans and queues image i + 1
// without waiting for image i (the copy into a slot waits on the device for
// the slot's previous image, and an image's small results land in the
// slot's pinned block, read once the stream has passed them), so a batch
// costs about max(copy, compute) per image and host jitter does not stall
// the copy engine.
pa_status find_obj_ring(pa_ctx *ctx, const pa_exp_param *e, int n_img, const pa_tree *trees,
                        int flip, const pa_classifier *const *cls, int n_cls, const float *desc,
                        const float *const *img_desc, int ny, int nx, int dim, const double *Tig,
                        int tig_shared, int H, int W, float *scores_out, const pa_ps_outputs *outs) {
  DeviceGuard dg(ctx->device);
  const int R = e->num_rotation_steps;
  const size_t per_img = (size_t)R * ny * nx * dim;
  const size_t bytes = per_img * sizeof(float);
  const int nslots = n_img < pa_ctx::kLandings ? n_img : pa_ctx::kLandings;
  if (!ctx->copy_stream) {
    if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_CUDA, "cannot create the copy stream");
    }
  }
  while ((int)ctx->ring_ev.size() < pa_ctx::kLandings) {
    cudaEvent_t ev;
    PA_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->ring_ev.push_back(ev);
  }
  while ((int)ctx->ring_done.size() < pa_ctx::kLandings) {
    cudaEvent_t ev;
    PA_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->ring_done.push_back(ev);
  }
  if (ctx->ring_cap < nslots * bytes) {
    PA_CK(cudaStreamSynchronize(ctx->copy_stream));
    PA_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->ring) cudaFree(ctx->ring);
    ctx->ring = nullptr;
    ctx->ring_cap = 0;
    if (cudaMalloc(&ctx->ring, nslots * bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes for the input ring", nslots * bytes);
    }
    ctx->ring_cap = nslots * bytes;
  }
  // the copy stream starts behind everything queued so far on the main stream
  PA_CK(cudaEventRecord(ctx->ring_done[0], ctx->stream));
  PA_CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ring_done[0], 0));
  auto issue = [&](int i) -> pa_status {
    const int k = i % nslots;
    const float *src = img_desc ? img_desc[i] : desc + i * per_img;
    PA_CK(cudaMemcpyAsync(ctx->ring + k * bytes, src, bytes, cudaMemcpyHostToDevice,
                          ctx->copy_stream));
    PA_CK(cudaEventRecord(ctx->ring_ev[k], ctx->copy_stream));
    return PA_OK;
  };
  std::vector<PendingImage> pend(nslots);
  auto drain = [&]() {  // leaves both streams idle after an error
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamSynchronize(ctx->stream);
  };
  pa_status result = PA_OK;
  // completes the image in slot k; NUMERIC is reported at the end, as the
  // images after it still run
  auto complete = [&](int k) -> pa_status {
    PendingImage &pi = pend[k];
    pi.busy = false;
    PA_CK(cudaEventSynchronize(ctx->ring_done[k]));
    const pa_status st = finish_complete(ctx, e, pi.pl, pi.outs, pi.rb);
    if (st == PA_ERR_NUMERIC) {
      result = st;
      return PA_OK;
    }
    return st;
  };
  for (int i = 0; i < nslots; ++i)
    if (pa_status st = issue(i)) {
      drain();
      return st;
    }
  for (int i = 0; i < n_img; ++i) {
    const int k = i % nslots;
    if (pend[k].busy)
      if (pa_status st = complete(k)) {
        drain();
        return st;
      }
    PA_CK(cudaStreamWaitEvent(ctx->stream, ctx->ring_ev[k], 0));
    pend[k].slot = k;
    pa_status st = find_obj_core(ctx, e, 1, &trees[i], flip, cls, n_cls,
                                 reinterpret_cast<const float *>(ctx->ring + k * bytes), nullptr,
                                 PA_MEM_DEVICE, ny, nx, dim, Tig, tig_shared, H, W, scores_out,
                                 (int64_t)i * R, (int64_t)n_img * R, &outs[i], PA_MEM_HOST,
                                 &pend[k]);
    if (st) {
      drain();
      return st;
    }
    pend[k].busy = true;
    PA_CK(cudaEventRecord(ctx->ring_done[k], ctx->stream));
    // slot k takes image i + nslots once image i has been computed
    if (i + nslots < n_img) {
      PA_CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ring_done[k], 0));
      if (pa_status s2 = issue(i + nslots)) {
        drain();
        return s2;
      }
    }
  }
  PA_CK(cudaStreamSynchronize(ctx->copy_stream));
  if (pa_status st = sync_ctx(ctx)) return st;
  for (int i = std::max(0, n_img - nslots); i < n_img; ++i)
    if (pend[i % nslots].busy)
      if (pa_status st = complete(i % nslots)) return st;
  return result;
}

pa_status find_obj_impl(pa_ctx *ctx, const pa_exp_param *e, int n_img, const pa_tree *trees,
                        int flip, const pa_classifier *const *cls, int n_cls, const float *desc,
                        int ny, int nx, int dim, const double *Tig, int tig_shared, int H, int W,
                        float *scores_out, const pa_ps_outputs *outs, int mem) {
  if (!exp_ok(e)) return fail(ctx, PA_ERR_INVALID, "invalid experiment parameters");
  if (n_scales(e) != 1)
    return fail(ctx, PA_ERR_UNSUPPORTED,
                "the descriptors are one scale; pa_find_obj_scales takes several");
  if (n_img < 1 || !trees || !desc || !Tig || !outs || ny < 1 || nx < 1 || dim < 1 || H < 1 ||
      W < 1 || H > 32767 || W > 32767)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  if (mem == PA_MEM_HOST && n_img > 1)
    return find_obj_ring(ctx, e, n_img, trees, flip, cls, n_cls, desc, nullptr, ny, nx, dim, Tig,
                         tig_shared, H, W, scores_out, outs);
  return find_obj_core(ctx, e, n_img, trees, flip, cls, n_cls, desc, nullptr, mem, ny, nx, dim,
                       Tig, tig_shared, H, W, scores_out, 0,
                       (int64_t)n_img * e->num_rotation_steps, outs, mem);
}

}  // namespace

// ==========================================================================
// C-ABI
// ==========================================================================
// ------------------------------------------------------------------------
// pa_find_obj_queue: waves of images, the message passing of a wave in one
// persistent launch (k_ps_queue).
// ------------------------------------------------------------------------
namespace {

struct QGroup {
  std::vector<int> idx;  // images of the call
  std::vector<pa_tree> trees;
  std::vector<pa_ps_outputs> outs;
  std::vector<const float *> desc;
  std::vector<std::vector<Joint>> joints;
  std::vector<float *> marg_out, rp_out;
  const pa_image *f = nullptr;
  PsPlan pl;  // the plan of the current pass
  StumpPart *sp = nullptr;
  const float *const *fields = nullptr;
  bool fields_al = true;
  float *scores = nullptr;
  const RankTables *rk = nullptr;  // rank form of the stump test, if the set qualifies
  uint32_t *ranks = nullptr;
  UnaryMap *umaps = nullptr;
  int usep = 0;
  Readback rb;  // where the group's small results land
};

// Plans one group (images of one shape) into b; `proto` carries the sizes
// and flags between the dry and the real pass.
pa_status plan_queue_group(pa_ctx *ctx, Builder &b, QGroup &g, const PsPlan &proto,
                           const pa_classifier *const *cls, int n_cls) {
  const pa_image &f = *g.f;
  const pa_exp_param *e = f.ep;
  const int n = (int)g.idx.size(), R = e->num_rotation_steps, P = proto.P;
  const int64_t G = (int64_t)f.ny * f.nx, n_fields = (int64_t)n * R;
  g.pl = proto;
  g.sp = plan_stumps(b, cls, n_cls);
  std::vector<const float *> fptr;
  g.fields_al = true;
  for (int i = 0; i < n; ++i)
    for (int r = 0; r < R; ++r) {
      fptr.push_back(g.desc[i] + (size_t)r * G * f.dim);
      g.fields_al = g.fields_al && ((uintptr_t)fptr.back() & 15) == 0;
    }
  g.fields = b.param(fptr.data(), fptr.size());
  g.scores = b.scratch<float>((size_t)n_cls * n_fields * G);
  g.rk = rank_tables(ctx, cls, n_cls);
  g.ranks = g.rk ? b.scratch<uint32_t>(rank_bytes(f.dim, G, (int)n_fields) / 4) : nullptr;
  plan_ps(b, g.pl, e, g.joints, g.marg_out.data(), g.rp_out.data());
  plan_marg_ptrs(b, g.pl);
  plan_localmax(b, g.pl, e, g.outs.data());
  std::vector<std::vector<float *>> uouts(n, std::vector<float *>(P, nullptr));
  for (int i = 0; i < n && !b.dry; ++i)
    for (int p = 0; p < P; ++p) uouts[i][p] = g.pl.im[i].U[p];
  return plan_unary(ctx, b, f.Tig, f.tig_shared, n, P, R, f.ny, f.nx, f.H, f.W, !e->interpolate,
                    g.scores, n_fields, uouts, g.pl.sc.upright, g.pl.sc.root,
                    e->strip_border_detections, g.pl.umax, e, &g.umaps, 1, &g.usep);
}

constexpr size_t kQSmemTwo = 112 * 1024;  // two queue CTAs per SM (228 KB less 1 KB each)

// Largest row-tile width (W itself, else a multiple of 352 outputs) whose
// layout fits `lim` bytes; 0 if none.
int queue_row_width(int R, int W, int kx, size_t lim) {
  if (ps_queue_smem_rows(R, W, kx) <= lim) return W;
  int best = 0;
  for (int c = 352; c < W; c += 352)
    if (ps_queue_smem_rows(R, c, kx) <= lim) best = c;
  return best;
}

// One wave.  PA_ERR_UNSUPPORTED: a message of the wave needs a path the
// queue does not run (the caller falls back to grouped launches).
pa_status queue_wave(pa_ctx *ctx, std::vector<QGroup> &groups, const pa_classifier *const *cls,
                     int n_cls, const pa_queue_opts &o) {
  cudaStream_t s = ctx->stream;
  std::vector<PsPlan> proto(groups.size());
  size_t n_jobs_max = 1;  // the gate
  for (size_t k = 0; k < groups.size(); ++k) {
    QGroup &g = groups[k];
    const pa_exp_param *e = g.f->ep;
    if (!e->use_pairwise) return PA_ERR_UNSUPPORTED;
    PsPlan &pl = proto[k];
    pl.tc_mode = false;
    pl.sparse_up = true;  // findObjectImageRotJoints passes bIsSparse = true
    pl.own_e2 = true;
    if (pa_status st = build_sched(ctx, &g.trees[0], pl.sc)) return st;
    if (pl.sc.ch[pl.sc.root].size() > (size_t)kQMaxDeps) return PA_ERR_UNSUPPORTED;
    for (size_t i = 1; i < g.trees.size(); ++i)
      if (!same_topology(&g.trees[0], &g.trees[i]))
        return fail(ctx, PA_ERR_INVALID, "image %d: tree topology differs", g.idx[i]);
    pl.B = (int)g.idx.size();
    pl.P = pl.sc.P;
    pl.R = e->num_rotation_steps;
    pl.H = g.f->H;
    pl.W = g.f->W;
    pl.N = (int64_t)pl.R * pl.H * pl.W;
    g.joints.assign(pl.B, {});
    for (int i = 0; i < pl.B; ++i)
      if (pa_status st = load_joints(ctx, &g.trees[i], g.f->flip, g.joints[i])) return st;
    if (n_cls < pl.P) return fail(ctx, PA_ERR_INVALID, "need at least n_parts classifiers");
    if (pa_status st = check_classifiers(ctx, cls, n_cls, g.f->dim)) return st;
    n_jobs_max += (size_t)pl.B * (4 * (pl.P - 1) + 1);
  }
  // pass 1 (dry), pass 2 (real): every group, then the queue's own words
  Builder b1;
  for (size_t k = 0; k < groups.size(); ++k)
    if (pa_status st = plan_queue_group(ctx, b1, groups[k], proto[k], cls, n_cls)) return st;
  b1.scratch<QJob>(n_jobs_max);
  b1.scratch<int>(n_jobs_max);
  b1.scratch<unsigned long long>(1);
  b1.scratch<int>(2);
  b1.scratch<unsigned long long>(16);
  if (pa_status st = ensure_arena(ctx, b1.total())) return st;
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  b.base = ctx->arena;
  for (size_t k = 0; k < groups.size(); ++k)
    if (pa_status st = plan_queue_group(ctx, b, groups[k], proto[k], cls, n_cls)) return st;
  QJob *d_jobs = b.scratch<QJob>(n_jobs_max);
  int *d_done = b.scratch<int>(n_jobs_max);
  unsigned long long *d_head = b.scratch<unsigned long long>(1);
  int *d_status = b.scratch<int>(2);
  unsigned long long *d_stats = b.scratch<unsigned long long>(16);
  if (b.blob.size() != b1.blob.size() || b.scratch_off != b1.scratch_off)
    return fail(ctx, PA_ERR_INVALID, "internal: plan size mismatch");
  for (QGroup &g : groups)
    for (auto *phs : {&g.pl.up, &g.pl.down})
      for (const PsPlan::Phase &ph : *phs)
        if (ph.n && (!ph.tma || ph.n_full || !ph.tc.empty())) return PA_ERR_UNSUPPORTED;

  // the jobs, in tree order: upward levels (rows, then columns), the roots,
  // downward levels
  std::vector<QJob> jobs;
  auto blank = []() {
    QJob j{};
    for (int d = 0; d < kQMaxDeps; ++d) j.dep[d] = -1;
    return j;
  };
  {
    QJob gate = blank();
    gate.type = QJOB_GATE;
    jobs.push_back(gate);
  }
  // key (group, image, child part, 0 up / 1 down, 0 rows / 1 cols) -> job
  std::map<std::tuple<int, int, int, int, int>, int> job_of;
  std::map<std::pair<int, int>, int> root_of;
  // tiles per queue item: one for a wave of few images (the tree's levels
  // leave most of the GPU to fill), up to four when many images overlap
  int wave_images = 0;
  for (QGroup &g : groups) wave_images += (int)g.idx.size();
  const int per = std::max(1, std::min(4, wave_images / 4));
  int maxd = 0;
  for (QGroup &g : groups) maxd = std::max(maxd, g.pl.sc.maxdepth);
  std::vector<std::pair<int, int>> tune_need;  // rows jobs whose width is still to choose
  auto emit_phase_jobs = [&](bool up, int depth, int kind) {
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      QGroup &g = groups[gi];
      const PsPlan &pl = g.pl;
      const auto &phs = up ? pl.up : pl.down;
      const int k = up ? pl.sc.maxdepth - depth : depth - 1;
      if (k < 0 || k >= (int)phs.size()) continue;
      const PsPlan::Phase &ph = phs[k];
      for (int q = 0; q < ph.n; ++q) {
        QJob j = blank();
        j.type = kind == 0 ? QJOB_ROWS : QJOB_COLS;
        j.md = ph.msgs + q;
        j.R = pl.R;
        j.H = pl.H;
        j.W = pl.W;
        if (kind == 0) {
          j.pad = ph.m_kx[q];
          j.cw = 0;  // chosen below
        } else {
          j.pad = ph.m_ky[q];
          j.nch = (pl.W + kColTileCols - 1) / kColTileCols;
          j.tiles = j.nch * pl.R * ((pl.H + kColBandRows - 1) / kColBandRows);
          j.per = per;
          j.n_items = (j.tiles + per - 1) / per;
        }
        job_of[std::make_tuple((int)gi, ph.m_img[q], ph.m_child[q], up ? 0 : 1, kind)] =
            (int)jobs.size();
        jobs.push_back(j);
      }
    }
  };
  for (int d = maxd; d >= 1; --d) {
    emit_phase_jobs(true, d, 0);
    emit_phase_jobs(true, d, 1);
  }
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const PsPlan &pl = groups[gi].pl;
    for (int i = 0; i < pl.B; ++i) {
      QJob j = blank();
      j.type = QJOB_ROOT;
      j.rd = pl.roots + i;
      j.cells = pl.N;
      j.tiles = (int)((pl.N + kQRootCells - 1) / kQRootCells);
      j.per = 1;
      j.n_items = j.tiles;
      root_of[{(int)gi, i}] = (int)jobs.size();
      jobs.push_back(j);
    }
  }
  for (int d = 1; d <= maxd; ++d) {
    emit_phase_jobs(false, d, 0);
    emit_phase_jobs(false, d, 1);
  }
  // dependencies
  for (auto &kv : job_of) {
    const int gi = std::get<0>(kv.first), i = std::get<1>(kv.first), c = std::get<2>(kv.first);
    const bool up = std::get<3>(kv.first) == 0;
    const int kind = std::get<4>(kv.first);
    const Sched &sc = groups[gi].pl.sc;
    QJob &j = jobs[kv.second];
    if (kind == 1) {  // columns after the message's rows
      j.dep[0] = job_of.at(std::make_tuple(gi, i, c, up ? 0 : 1, 0));
    } else if (up) {  // rows of c -> parent after c's belief is complete
      if (sc.ch[c].empty()) j.dep[0] = 0;
      else
        for (size_t k = 0; k < sc.ch[c].size() && k < (size_t)kQMaxDeps; ++k)
          j.dep[k] = job_of.at(std::make_tuple(gi, i, sc.ch[c][k], 0, 1));
    } else {  // rows of parent -> c after the parent's from-root belief
      int par = -1;
      for (int p = 0; p < sc.P; ++p)
        for (int ch : sc.ch[p])
          if (ch == c) par = p;
      j.dep[0] = par == sc.root ? root_of.at({gi, i})
                                : job_of.at(std::make_tuple(gi, i, par, 1, 1));
    }
  }
  for (auto &kv : root_of) {
    const Sched &sc = groups[kv.first.first].pl.sc;
    QJob &j = jobs[kv.second];
    if (sc.ch[sc.root].empty()) j.dep[0] = 0;
    for (size_t k = 0; k < sc.ch[sc.root].size(); ++k)
      j.dep[k] = job_of.at(std::make_tuple(kv.first.first, kv.first.second, sc.ch[sc.root][k], 0, 1));
  }

  // The per-group work before and after the queue (unaries; root marginal,
  // log-partition, local maxima and result copies) runs on up to kWorkers
  // side streams forked from the caller's stream and joined back into it.
  const int NS = std::min((int)groups.size(), pa_ctx::kWorkers);
  while ((int)ctx->side.size() < NS) {
    cudaStream_t st = nullptr;
    PA_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    ctx->side.push_back(st);
  }
  struct OnStream {  // ctx->stream set to a side stream for one group's launches
    pa_ctx *c;
    cudaStream_t keep;
    OnStream(pa_ctx *c_, cudaStream_t st) : c(c_), keep(c_->stream) { c->stream = st; }
    ~OnStream() { c->stream = keep; }
  };
  auto fork = [&]() -> pa_status {
    cudaEvent_t ev = take_event(ctx);
    PA_CK(cudaEventRecord(ev, s));
    for (int k = 0; k < NS; ++k) PA_CK(cudaStreamWaitEvent(ctx->side[k], ev, 0));
    ctx->pool.push_back(ev);  // a wait binds the record made before it
    return PA_OK;
  };
  auto join = [&]() -> pa_status {
    for (int k = 0; k < NS; ++k) {
      cudaEvent_t ev = take_event(ctx);
      PA_CK(cudaEventRecord(ev, ctx->side[k]));
      PA_CK(cudaStreamWaitEvent(s, ev, 0));
      ctx->pool.push_back(ev);
    }
    return PA_OK;
  };

  // unaries of every group (the inputs of the first messages)
  if (pa_status st = upload_blob(ctx, b)) return st;
  for (QGroup &g : groups)
    if (pa_status st = init_slots(ctx, g.pl)) return st;
  if (pa_status st = fork()) return st;
  {
    const std::vector<char> ff = fast_flags(cls, n_cls);
    const std::vector<int> ns = stump_counts(cls, n_cls);
    for (size_t k = 0; k < groups.size(); ++k) {
      QGroup &g = groups[k];
      const pa_image &f = *g.f;
      const int n = (int)g.idx.size(), R = g.pl.R;
      const int64_t G = (int64_t)f.ny * f.nx, n_fields = (int64_t)n * R;
      OnStream on(ctx, ctx->side[k % NS]);
      cudaStream_t gs = ctx->stream;
      if (g.rk)
      {
        PA_LAUNCH("stump_ranks", launch_rank_buckets(*g.rk, g.desc[0], g.fields, g.fields_al, G,
                                                     (int)n_fields, g.ranks, gs));
        PA_LAUNCH("stump_votes", launch_rank_votes(*g.rk, G, (int)n_fields, 1, g.scores, g.ranks,
                                                   g.pl.err, gs));
      } else
        PA_LAUNCH("score_grids", launch_score_grids(g.sp, (const bool *)ff.data(), ns.data(), n_cls,
                                                    g.desc[0], g.fields, g.fields_al, G,
                                                    (int)n_fields, f.dim, 1, g.scores, gs));
      PA_LAUNCH_N("unary_maps", unary_launches(!f.ep->interpolate, g.usep),
                  launch_unary_maps(g.umaps, n * g.pl.P * R, f.ny, f.nx, f.H, f.W,
                                    !f.ep->interpolate, g.usep & kUnarySeparable,
                                    g.usep & kUnaryOrdered, gs));
      if (g.pl.n_msgs_total > 0)
        PA_LAUNCH_N("shift_tables", 2,
                    launch_shift_tables(g.pl.shifts, g.pl.n_msgs_total, R, f.H, f.W, g.pl.tables,
                                        g.pl.sdesc, gs));
    }
  }
  if (pa_status st = join()) return st;

  // row-tile widths: measured once per shape class (R, W, kx) on a message
  // whose input (a leaf's unary) is ready, among the widths that fit
  std::vector<std::pair<int, int>> cls_job;  // first leaf-upward rows job of each new class
  for (auto &kv : job_of) {
    if (std::get<4>(kv.first) != 0) continue;
    QJob &j = jobs[kv.second];
    const auto key = std::make_tuple(j.R, j.W, j.pad);
    auto it = ctx->row_tile.find(key);
    if (it != ctx->row_tile.end()) {
      j.cw = it->second;
      continue;
    }
    const bool leaf_up = std::get<3>(kv.first) == 0 && j.dep[0] == 0;
    if (o.autotune && leaf_up) {
      bool have = false;
      for (auto &cj : cls_job)
        if (jobs[cj.second].R == j.R && jobs[cj.second].W == j.W && jobs[cj.second].pad == j.pad) have = true;
      if (!have) cls_job.push_back({0, kv.second});
    }
  }
  cudaEvent_t t0 = take_event(ctx), t1 = take_event(ctx);
  for (auto &cj : cls_job) {
    const QJob &j = jobs[cj.second];
    std::vector<int> cand;
    for (size_t lim : {kQSmemTwo, (size_t)227 * 1024}) {
      for (int c : {j.W, 704, 352})
        if (c <= j.W && ps_queue_smem_rows(j.R, c, j.pad) <= lim &&
            std::find(cand.begin(), cand.end(), c) == cand.end())
          cand.push_back(c);
      if (!cand.empty()) break;
    }
    int best = 0;
    float best_ms = 0.f;
    for (int c : cand) {
      for (int rep = 0; rep < 2; ++rep) {
        PA_CK(cudaEventRecord(t0, s));
        PA_CK(launch_msg_rows_cw(j.md, 1, j.R, j.H, j.W, j.pad, c, groups[0].pl.err, s));
        PA_CK(cudaEventRecord(t1, s));
      }
      PA_CK(cudaEventSynchronize(t1));
      float ms = 0.f;
      PA_CK(cudaEventElapsedTime(&ms, t0, t1));
      if (!best || ms < best_ms) {
        best = c;
        best_ms = ms;
      }
    }
    if (best) ctx->row_tile[std::make_tuple(j.R, j.W, j.pad)] = best;
  }
  ctx->pool.push_back(t0);
  ctx->pool.push_back(t1);
  size_t smem = 0;
  for (auto &kv : job_of) {
    QJob &j = jobs[kv.second];
    if (std::get<4>(kv.first) == 0) {
      if (!j.cw) {
        auto it = ctx->row_tile.find(std::make_tuple(j.R, j.W, j.pad));
        j.cw = it != ctx->row_tile.end() ? it->second : queue_row_width(j.R, j.W, j.pad, kQSmemTwo);
        if (!j.cw) j.cw = queue_row_width(j.R, j.W, j.pad, (size_t)227 * 1024);
        if (!j.cw) return PA_ERR_UNSUPPORTED;
      }
      j.nch = (j.W + j.cw - 1) / j.cw;
      j.tiles = j.H * j.nch;
      j.per = per;
      j.n_items = (j.tiles + per - 1) / per;
      smem = std::max(smem, ps_queue_smem_rows(j.R, j.cw, j.pad));
    } else {
      smem = std::max(smem, ps_queue_smem_cols(j.pad));
    }
  }
  long long n_items = 0;
  for (QJob &j : jobs) {
    j.first = n_items;
    n_items += j.n_items;
  }
  if (jobs.size() > n_jobs_max) return fail(ctx, PA_ERR_INVALID, "internal: job count");
  if (pa_status st = upload_to(ctx, d_jobs, jobs.data(), jobs.size() * sizeof(QJob))) return st;
  PA_CK(cudaMemsetAsync(d_done, 0, jobs.size() * sizeof(int), s));
  PA_CK(cudaMemsetAsync(d_head, 0, sizeof(unsigned long long), s));
  PA_CK(cudaMemsetAsync(d_status, 0, 2 * sizeof(int), s));
  // the host opens the start gate (the jobs of the leaves wait for it)
  if (!o.hold_start) PA_LAUNCH("fill", launch_fill_int(d_done, 1, 1, s));
  const long long wait_ns =
      (long long)((o.wait_timeout_ms > 0 ? o.wait_timeout_ms : 20000.0) * 1e6);
  int ctas = 0;
  // PA_QUEUE_STATS=1: per job type, time taking tiles, waiting and running
  // them (summed over CTAs), printed to stderr after each wave
  const char *want_stats = std::getenv("PA_QUEUE_STATS");
  const bool stats = want_stats && want_stats[0] == '1';
  if (stats) PA_CK(cudaMemsetAsync(d_stats, 0, 16 * sizeof(unsigned long long), s));
  PA_LAUNCH("ps_queue", launch_ps_queue(d_jobs, (int)jobs.size(), n_items, d_head, d_done, d_status,
                                        groups[0].pl.err, wait_ns, smem, &ctas,
                                        stats ? d_stats : nullptr, s));
  // the status word and the first group's error word (the tiles' error
  // bits) land in pinned memory, read when the wave is finished
  if (!ctx->qwords) {
    if (cudaMallocHost(&ctx->qwords, 4 * sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate pinned status words");
    }
  }
  PA_CK(cudaMemcpyAsync(ctx->qwords, d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  PA_CK(cudaMemcpyAsync(ctx->qwords + 1, groups[0].pl.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (stats) {
    PA_CK(cudaStreamSynchronize(s));
    unsigned long long h[16];
    PA_CK(cudaMemcpy(h, d_stats, sizeof h, cudaMemcpyDeviceToHost));
    static const char *names[4] = {"rows", "cols", "root", "rows48"};
    std::fprintf(stderr, "ps_queue: %d CTAs, %zu jobs, %lld items of %d tiles, smem %zu\n", ctas, jobs.size(),
                 n_items, per, smem);
    for (int t = 0; t < 4; ++t)
      if (h[4 * t + 3])
        std::fprintf(stderr, "  %-4s tiles %8llu  take %7.2f us  wait %7.2f us  run %7.2f us\n",
                     names[t], h[4 * t + 3], 1e-3 * h[4 * t] / h[4 * t + 3],
                     1e-3 * h[4 * t + 1] / h[4 * t + 3], 1e-3 * h[4 * t + 2] / h[4 * t + 3]);
  }
  // tails: each group's results land in its own pinned block (read by
  // queue_wave_finish after one sync)
  if (ctx->land.size() < groups.size()) ctx->land.resize(groups.size());
  if (pa_status st = fork()) return st;
  for (size_t k = 0; k < groups.size(); ++k) {
    QGroup &g = groups[k];
    OnStream on(ctx, ctx->side[k % NS]);
    if (pa_status st = run_ps_tail(ctx, g.f->ep, g.pl)) return st;
    if (pa_status st = finish_enqueue(ctx, g.f->ep, g.pl, g.outs.data(), PA_MEM_DEVICE, (int)k, g.rb))
      return st;
  }
  return join();
}

// Waits for a wave queued by queue_wave on ctx and decodes its results.
pa_status queue_wave_finish(pa_ctx *ctx, std::vector<QGroup> &groups, const pa_queue_opts &o) {
  if (pa_status st = sync_ctx(ctx)) return st;
  if (ctx->qwords[0] & 1)
    return fail(ctx, PA_ERR_TIMEOUT, "a queue dependency wait ran out (%.0f ms)",
                o.wait_timeout_ms > 0 ? o.wait_timeout_ms : 20000.0);
  // a tile's error bits went to the first group's word: they count for all
  const int err0 = ctx->qwords[1];
  pa_status result = PA_OK;
  for (size_t k = 0; k < groups.size(); ++k) {
    QGroup &g = groups[k];
    if (k > 0) *g.rb.err |= err0;
    const pa_status st = finish_complete(ctx, g.f->ep, g.pl, g.outs.data(), g.rb);
    if (st == PA_ERR_NUMERIC) result = st;
    else if (st) return st;
  }
  return result;
}

}  // namespace

extern "C" {

const char *pa_status_string(pa_status s) {
  switch (s) {
    case PA_OK: return "ok";
    case PA_ERR_INVALID: return "invalid argument";
    case PA_ERR_UNSUPPORTED: return "unsupported";
    case PA_ERR_CUDA: return "CUDA error";
    case PA_ERR_NOMEM: return "out of memory";
    case PA_ERR_NUMERIC: return "numeric overflow";
    case PA_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

void pa_exp_param_default(pa_exp_param *p) {
  if (!p) return;
  p->num_rotation_steps = 48;
  p->min_part_rotation = -180.f;
  p->max_part_rotation = 180.f;
  p->min_object_scale = 1.f;
  p->max_object_scale = 1.f;
  p->strip_border_detections = 0.f;
  p->roi_save_num_samples = 1000;
  p->use_pairwise = 1;
  p->interpolate = 0;
  p->num_scale_steps = 1;
}

pa_status pa_ctx_create(int device, pa_ctx **out) try {
  if (!out) return PA_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return PA_ERR_CUDA;
  }
  std::unique_ptr<pa_ctx> c(new pa_ctx);
  c->device = device;
  DeviceGuard dg(device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return PA_ERR_CUDA;
  }
  c->own_stream = true;
  *out = c.release();
  return PA_OK;
} catch (const std::bad_alloc &) {
  return PA_ERR_NOMEM;
} catch (...) {
  return PA_ERR_INVALID;
}

pa_status pa_ctx_destroy(pa_ctx *ctx) try {
  if (!ctx) return PA_OK;
  for (pa_ctx *w : ctx->workers) pa_ctx_destroy(w);
  ctx->workers.clear();
  {
    DeviceGuard dg(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    resolve_timing(ctx);
    for (cudaEvent_t e : ctx->pool) cudaEventDestroy(e);
    if (ctx->arena) cudaFree(ctx->arena);
    if (ctx->scales_buf) cudaFree(ctx->scales_buf);
    for (auto &sg : ctx->stage) {
      if (sg.p) cudaFreeHost(sg.p);
      if (sg.done) cudaEventDestroy(sg.done);
    }
    for (auto &ld : ctx->land)
      if (ld.p) cudaFreeHost(ld.p);
    for (cudaEvent_t e : ctx->ring_done) cudaEventDestroy(e);
    for (cudaStream_t st : ctx->side) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
    for (auto &kv : ctx->rank_sets)
      if (kv.second.mem) cudaFree(kv.second.mem);
    if (ctx->qwords) cudaFreeHost(ctx->qwords);
    if (ctx->copy_stream) {
      cudaStreamSynchronize(ctx->copy_stream);
      cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->ring) cudaFree(ctx->ring);
    for (cudaEvent_t e : ctx->ring_ev) cudaEventDestroy(e);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_ctx_set_stream(pa_ctx *ctx, void *stream) try {
  if (!ctx) return PA_ERR_INVALID;
  DeviceGuard dg(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = (cudaStream_t)stream;
  ctx->own_stream = false;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_ctx_set_message_math(pa_ctx *ctx, int mode) try {
  if (!ctx) return PA_ERR_INVALID;
  if (mode != PA_MSG_FP32 && mode != PA_MSG_BF16_TENSOR)
    return fail(ctx, PA_ERR_INVALID, "unknown message math %d", mode);
  ctx->msg_math = mode;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_ctx_synchronize(pa_ctx *ctx) try {
  if (!ctx) return PA_ERR_INVALID;
  DeviceGuard dg(ctx->device);
  PA_CK(cudaStreamSynchronize(ctx->stream));
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

const char *pa_last_error(const pa_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

uint64_t pa_ctx_kernel_launches(const pa_ctx *ctx) { return ctx ? ctx->launches : 0; }

pa_status pa_ctx_enable_timing(pa_ctx *ctx, int on) try {
  if (!ctx) return PA_ERR_INVALID;
  DeviceGuard dg(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  resolve_timing(ctx);
  ctx->timing = on != 0;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_ctx_timing_reset(pa_ctx *ctx) try {
  if (!ctx) return PA_ERR_INVALID;
  DeviceGuard dg(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  resolve_timing(ctx);
  ctx->times.clear();
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

int pa_ctx_timing_count(pa_ctx *ctx) {
  if (!ctx) return 0;
  ctx->names.clear();
  for (auto &kv : ctx->times) ctx->names.push_back(kv.first);
  return (int)ctx->names.size();
}

pa_status pa_ctx_timing_get(pa_ctx *ctx, int i, const char **name, double *total_ms,
                            uint64_t *launches) try {
  if (!ctx || i < 0 || i >= (int)ctx->names.size()) return PA_ERR_INVALID;
  const auto &acc = ctx->times[ctx->names[i]];
  if (name) *name = ctx->names[i].c_str();
  if (total_ms) *total_ms = acc.ms;
  if (launches) *launches = acc.n;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_classifier_create(pa_ctx *ctx, int dim, const pa_stump *stumps, int n_stumps,
                               pa_classifier **out) try {
  if (!ctx || !out) return PA_ERR_INVALID;
  *out = nullptr;
  if (dim < 1 || n_stumps < 1 || !stumps)
    return fail(ctx, PA_ERR_INVALID, "classifier needs dim >= 1 and stumps");
  std::vector<float4> host(n_stumps), fast(n_stumps);
  float sum_alpha = 0.f;  // operator>>, AdaBoost.cc:327-331
  bool unit_polarity = true;
  for (int i = 0; i < n_stumps; ++i) {
    if (stumps[i].f < 0 || stumps[i].f >= dim)
      return fail(ctx, PA_ERR_INVALID, "stump %d: feature %d outside [0,%d)", i, stumps[i].f, dim);
    float fbits;
    std::memcpy(&fbits, &stumps[i].f, 4);
    const float p = stumps[i].p, th = stumps[i].theta, a = stumps[i].alpha;
    // theta * p is the right-hand side of the stump test (AdaBoost.h:156);
    // the device compares v * p against this same float product.
    host[i] = make_float4(fbits, p, th * p, a);
    // p = +1: v < theta; p = -1: v > theta == !(v < nextafter(theta, +inf))
    if (std::isnan(th)) unit_polarity = false;
    else if (p == 1.0f) fast[i] = make_float4(fbits, th, a, 0.f);
    else if (p == -1.0f) fast[i] = make_float4(fbits, std::nextafter(th, INFINITY), -a, 0.f);
    else unit_polarity = false;
    sum_alpha += a;
  }
  DeviceGuard dg(ctx->device);
  std::unique_ptr<pa_classifier> c(new pa_classifier);
  static std::atomic<uint64_t> next_id{1};
  c->id = next_id.fetch_add(1);
  c->dim = dim;
  c->n = n_stumps;
  c->sum_alpha = sum_alpha;
  if (cudaMalloc(&c->d, sizeof(float4) * n_stumps) != cudaSuccess) {
    cudaGetLastError();
    return fail(ctx, PA_ERR_NOMEM, "cannot allocate stump table");
  }
  PA_CK(cudaMemcpy(c->d, host.data(), sizeof(float4) * n_stumps, cudaMemcpyHostToDevice));
  if (unit_polarity) {
    if (cudaMalloc(&c->fast, sizeof(float4) * n_stumps) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(c->d);
      return fail(ctx, PA_ERR_NOMEM, "cannot allocate stump table");
    }
    PA_CK(cudaMemcpy(c->fast, fast.data(), sizeof(float4) * n_stumps, cudaMemcpyHostToDevice));
    c->fast_h = fast;
    // packed copy; stumps past n are {t = -inf, a = +0}: their vote -0 leaves
    // the running sum (which starts at +0 and is never -0) unchanged
    if (dim <= 65536) {
      const int npad = (n_stumps + 7) / 8 * 8;
      std::vector<uint16_t> f16(npad, 0);
      std::vector<float> ta(2 * (size_t)npad);
      for (int i = 0; i < npad; ++i) {
        if (i < n_stumps) {
          f16[i] = (uint16_t)stumps[i].f;
          ta[2 * i] = fast[i].y;
          ta[2 * i + 1] = fast[i].z;
        } else {
          ta[2 * i] = -INFINITY;
          ta[2 * i + 1] = 0.f;
        }
      }
      const size_t fb = (size_t)npad * 2, tb = (size_t)npad * 8;
      if (cudaMalloc(&c->packed, fb + tb) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->d);
        cudaFree(c->fast);
        return fail(ctx, PA_ERR_NOMEM, "cannot allocate stump table");
      }
      PA_CK(cudaMemcpy(c->packed, f16.data(), fb, cudaMemcpyHostToDevice));
      PA_CK(cudaMemcpy(c->packed + fb, ta.data(), tb, cudaMemcpyHostToDevice));
      c->npad = npad;
    }
  }
  *out = c.release();
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_classifier_parse(pa_ctx *ctx, const char *text, size_t len, pa_classifier **out) try {
  if (!ctx || !text || !out) return PA_ERR_INVALID;
  std::string s(text, len);
  const char *p = s.c_str();
  char *end = nullptr;
  auto next_num = [&](double &v) -> bool {
    v = std::strtod(p, &end);
    if (end == p) return false;
    p = end;
    return true;
  };
  double dv, nv;
  if (!next_num(dv) || !next_num(nv) || !(dv >= 1 && dv <= (1 << 24)) ||
      !(nv >= 1 && nv <= (1 << 24)))
    return fail(ctx, PA_ERR_INVALID, "classifier text: missing or out-of-range D / number of stumps");
  const int D = (int)dv, ns = (int)nv;
  // every stump takes at least 10 characters ("f p a j t" with separators):
  // a count the text cannot hold is rejected before anything is allocated
  if ((size_t)ns > len / 10 + 1)
    return fail(ctx, PA_ERR_INVALID, "classifier text: %d stumps announced, the text is shorter", ns);
  std::vector<pa_stump> st(ns);
  for (int i = 0; i < ns; ++i) {
    double f, pp, a, j, th;
    if (!next_num(f) || !next_num(pp) || !next_num(a) || !next_num(j) || !next_num(th))
      return fail(ctx, PA_ERR_INVALID, "classifier text: stump %d truncated", i);
    if (!(f >= 0 && f < D))
      return fail(ctx, PA_ERR_INVALID, "classifier text: stump %d: feature index out of range", i);
    st[i].f = (int32_t)f;
    st[i].p = (float)pp;
    st[i].alpha = (float)a;
    st[i].theta = (float)th;
  }
  return pa_classifier_create(ctx, D, st.data(), ns, out);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_classifier_destroy(pa_ctx *ctx, pa_classifier *cls) try {
  if (!cls) return PA_OK;
  if (ctx) {
    DeviceGuard dg(ctx->device);
    cudaFree(cls->d);
    if (cls->fast) cudaFree(cls->fast);
    if (cls->packed) cudaFree(cls->packed);
  } else {
    cudaFree(cls->d);
    if (cls->fast) cudaFree(cls->fast);
    if (cls->packed) cudaFree(cls->packed);
  }
  delete cls;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_classifier_info(const pa_classifier *cls, int *dim, int *n_stumps, float *sum_alpha) try {
  if (!cls) return PA_ERR_INVALID;
  if (dim) *dim = cls->dim;
  if (n_stumps) *n_stumps = cls->n;
  if (sum_alpha) *sum_alpha = cls->sum_alpha;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return PA_ERR_NOMEM;
} catch (...) {
  return PA_ERR_INVALID;
}

namespace {

// pa_score_grids with the descriptors in in_mem and the scores in out_mem.
pa_status score_grids_impl(pa_ctx *ctx, const pa_classifier *const *cls, int n_parts,
                           const float *desc, int in_mem, int n_fields, int ny, int nx, int dim,
                           int normalize, float *scores, int out_mem) {
  pa_status st = check_classifiers(ctx, cls, n_parts, dim);
  if (st) return st;
  DeviceGuard dg(ctx->device);
  const int64_t G = (int64_t)ny * nx;
  const size_t din = (size_t)n_fields * G * dim, dout = (size_t)n_parts * n_fields * G;
  const RankTables *rk = rank_tables(ctx, cls, n_parts);
  Builder b1;
  plan_stumps(b1, cls, n_parts);
  if (in_mem == PA_MEM_HOST) b1.scratch<float>(din);
  if (out_mem == PA_MEM_HOST) b1.scratch<float>(dout);
  if (rk) {
    b1.scratch<uint32_t>(rank_bytes(dim, G, n_fields) / 4);
    b1.scratch<int>(1);
  }
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  st = ensure_arena(ctx, b1.total());
  if (st) return st;
  b.base = ctx->arena;
  StumpPart *sp = plan_stumps(b, cls, n_parts);
  const float *d_in = in_mem == PA_MEM_HOST ? b.scratch<float>(din) : desc;
  float *d_out = out_mem == PA_MEM_HOST ? b.scratch<float>(dout) : scores;
  uint32_t *ranks = rk ? b.scratch<uint32_t>(rank_bytes(dim, G, n_fields) / 4) : nullptr;
  int *d_err = rk ? b.scratch<int>(1) : nullptr;
  st = upload_blob(ctx, b);
  if (st) return st;
  if (in_mem == PA_MEM_HOST) {
    st = copy_in(ctx, (void *)d_in, desc, din * sizeof(float), in_mem);
    if (st) return st;
  }
  int errflag = 0;
  if (rk) {
    PA_CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
    PA_LAUNCH("stump_ranks", launch_rank_buckets(*rk, d_in, nullptr, ((uintptr_t)d_in & 15) == 0, G,
                                                 n_fields, ranks, ctx->stream));
    PA_LAUNCH("stump_votes", launch_rank_votes(*rk, G, n_fields, normalize, d_out, ranks, d_err,
                                               ctx->stream));
    PA_CK(cudaMemcpyAsync(&errflag, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    const std::vector<char> ff = fast_flags(cls, n_parts);
    const std::vector<int> ns = stump_counts(cls, n_parts);
    PA_LAUNCH("score_grids", launch_score_grids(sp, (const bool *)ff.data(), ns.data(), n_parts, d_in, nullptr, false, G,
                                                n_fields, dim, normalize, d_out, ctx->stream));
  }
  if (out_mem == PA_MEM_HOST)
    PA_CK(cudaMemcpyAsync(scores, d_out, dout * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  st = sync_ctx(ctx);
  if (st) return st;
  if (errflag) return fail(ctx, PA_ERR_CUDA, "rank tile copy did not complete (error bits %d)", errflag);
  return PA_OK;
}

}  // namespace

pa_status pa_score_grids(pa_ctx *ctx, const pa_classifier *const *cls, int n_parts,
                         const float *desc, int n_fields, int ny, int nx, int dim, int normalize,
                         float *scores, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!desc || !scores || n_fields < 1 || ny < 1 || nx < 1 || dim < 1)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  return score_grids_impl(ctx, cls, n_parts, desc, mem, n_fields, ny, nx, dim, normalize, scores,
                          mem);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

// ------------------------------------------------------------------------
// SHAPEv5 descriptor grid (computeDescriptorGrid, partdetect_aux.cpp:77-190)
// ------------------------------------------------------------------------
namespace {

// FeatureGrid(img_width, img_height, x_axis, y_axis, desc_step, _)
// (libPartDetect/FeatureGrid.cpp:22-97): the image's bounding box in the
// grid frame, from the 2 x 2 inverse of boost_math::inv (boost_math.hpp:103-110).
bool feature_grid(int w, int h, const double *ax, const double *ay, double step, double *rect,
                  int *nx, int *ny) {
  const double m00 = ax[0], m01 = ay[0], m10 = ax[1], m11 = ay[1];
  const double D = m00 * m11 - m10 * m01;
  if (!(D != 0.0) || !std::isfinite(D)) return false;
  const double t00 = m11 / D, t01 = -m01 / D, t10 = -m10 / D, t11 = m00 / D;
  const double cx[4] = {0, (double)w, (double)w, 0}, cy[4] = {0, 0, (double)h, (double)h};
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
  const double fx = std::floor(((mxx - mnx + 1) / step)) + 1;
  const double fy = std::floor(((mxy - mny + 1) / step)) + 1;
  if (!(fx >= 1 && fy >= 1 && fx * fy <= (double)(1 << 28))) return false;
  *nx = (int)fx;
  *ny = (int)fy;
  return true;
}

// initPatchMask(21) (FeatureDescriptor.cpp:118-137) and precompute_patch_idx
// (ShapeDescriptor.cpp:42-64) with the reference's float / double types.
void patch_tables(DescTables &t) {
  constexpr int P = 21, center = P >> 1;
  constexpr double m2pi = 6.2831853072;  // M_2PI, libKMA2/gauss_iir/gauss_iir.h:21
  std::memset(&t, 0, sizeof t);
  const float radius = center * center;
  const float sigma = 0.9 * radius;
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) {
      const float disq = (i - center) * (i - center) + (j - center) * (j - center);
      t.mask[j * P + i] = disq < radius ? std::exp(-disq / sigma) : 0.f;
    }
  const float cspacing = 4 / (m2pi);  // ScSize / M_2PI
  for (int i = -center; i <= center; ++i)
    for (int j = -center; j <= center; ++j) {
      const double lcpos = (M_PI + std::atan2((double)i, (double)j)) * cspacing;
      const double lrpos = std::log(1 + std::sqrt((float)i * i + j * j) / center) * 3;  // SrSize
      const int k = (center + j) * P + (center + i);
      t.lc[k] = (float)lcpos;
      t.lr[k] = (float)lrpos;
      t.inrange[k] = (lrpos > -1.0 && lrpos < (float)3 && lcpos > -1.0 && lcpos < (float)4) ? 1 : 0;
    }
}

// set_nii_and_dii + set_smooth_coefficients (libKMA2/gauss_iir/gauss_iir.cpp:
// 47-120): Deriche's fourth-order recursive Gaussian of width sigma, float.
void smooth_coefficients(float sigma, float *coefs) {
  const float a0 = 1.68f, a1 = 3.735f, b0 = 1.783f, b1 = 1.723f, c0 = -0.6803f, c1 = -0.2598f,
              omega0 = 0.6318f, omega1 = 1.997f;
  using std::cos;
  using std::exp;
  using std::sin;
  coefs[0] = a0 + c0;
  coefs[1] = exp(-b1 / sigma) * (c1 * sin(omega1 / sigma) - (c0 + 2 * a0) * cos(omega1 / sigma)) +
             exp(-b0 / sigma) * (a1 * sin(omega0 / sigma) - (2 * c0 + a0) * cos(omega0 / sigma));
  coefs[2] = 2 * exp(-b0 / sigma - b1 / sigma) *
                 ((a0 + c0) * cos(omega1 / sigma) * cos(omega0 / sigma) -
                  cos(omega1 / sigma) * a1 * sin(omega0 / sigma) -
                  cos(omega0 / sigma) * c1 * sin(omega1 / sigma)) +
             c0 * exp(-2 * b0 / sigma) + a0 * exp(-2 * b1 / sigma);
  coefs[3] = exp(-b1 / sigma - 2 * b0 / sigma) * (c1 * sin(omega1 / sigma) - c0 * cos(omega1 / sigma)) +
             exp(-b0 / sigma - 2 * b1 / sigma) * (a1 * sin(omega0 / sigma) - a0 * cos(omega0 / sigma));
  coefs[8] = -2 * exp(-b1 / sigma) * cos(omega1 / sigma) - 2 * exp(-b0 / sigma) * cos(omega0 / sigma);
  coefs[9] = 4 * cos(omega1 / sigma) * cos(omega0 / sigma) * exp(-b0 / sigma - b1 / sigma) +
             exp(-2 * b1 / sigma) + exp(-2 * b0 / sigma);
  coefs[10] = -2 * cos(omega0 / sigma) * exp(-b0 / sigma - 2 * b1 / sigma) -
              2 * cos(omega1 / sigma) * exp(-b1 / sigma - 2 * b0 / sigma);
  coefs[11] = exp(-2 * b0 / sigma - 2 * b1 / sigma);
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

}  // namespace

namespace {

// The inside test of computeDescriptorGrid (partdetect_aux.cpp:128-130:
// imgpos >= desc_size + 1, imgpos <= x() - (desc_size + 1) in x()'s unsigned
// arithmetic) intersected with its region-of-interest test (:113-118,
// 140-145).  roi = {x, y, width, height} as QRect(x, y, width, height) holds
// it (right() = x + width - 1), or null for the QRect(0, 0, x() - 1, y() - 1)
// every default entry builds (:44-55), whose right() is x() - 2: that one is
// tested too, and bites when desc_size is 0.  Both tests skip a position the
// same way, so one box holds both.
void desc_bounds(DescGrid &g, int w, int h, int desc_size, const int *roi) {
  g.lo_x = g.lo_y = (double)(desc_size + 1);
  g.hi_x = (double)((unsigned)w - (unsigned)(desc_size + 1));
  g.hi_y = (double)((unsigned)h - (unsigned)(desc_size + 1));
  const long long l = roi ? roi[0] : 0, t = roi ? roi[1] : 0;
  const long long r = roi ? (long long)roi[0] + roi[2] - 1 : (long long)w - 2;
  const long long b = roi ? (long long)roi[1] + roi[3] - 1 : (long long)h - 2;
  if (l == 0 && r == (long long)w - 1 && t == 0 && b == (long long)h - 1) return;  // bTestRoi false
  g.lo_x = std::max(g.lo_x, (double)l);
  g.lo_y = std::max(g.lo_y, (double)t);
  g.hi_x = std::min(g.hi_x, (double)r);
  g.hi_y = std::min(g.hi_y, (double)b);
}

}  // namespace

pa_status pa_feature_grid_size(int img_w, int img_h, const double *x_axis, const double *y_axis,
                               double desc_step, int *nx, int *ny) try {
  if (img_w < 1 || img_h < 1 || !x_axis || !y_axis || !nx || !ny || !(desc_step > 0))
    return PA_ERR_INVALID;
  double rect[4];
  return feature_grid(img_w, img_h, x_axis, y_axis, desc_step, rect, nx, ny) ? PA_OK
                                                                              : PA_ERR_INVALID;
} catch (const std::bad_alloc &) {
  return PA_ERR_NOMEM;
} catch (...) {
  return PA_ERR_INVALID;
}

pa_status pa_descriptor_grid(pa_ctx *ctx, const float *image, int img_h, int img_w,
                             const double *x_axis, const double *y_axis, double desc_step,
                             int desc_size, float *cells, uint8_t *valid, int mem) {
  return pa_descriptor_grid_masked(ctx, image, img_h, img_w, x_axis, y_axis, desc_step,
                                   desc_size, nullptr, nullptr, cells, valid, mem);
}

pa_status pa_descriptor_grid_masked(pa_ctx *ctx, const float *image, int img_h, int img_w,
                                    const double *x_axis, const double *y_axis,
                                    double desc_step, int desc_size,
                                    const float *detection_mask, const int *roi, float *cells,
                                    uint8_t *valid, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!image || !cells || !valid || !x_axis || !y_axis || img_h < 2 || img_w < 2 ||
      !(desc_step > 0) || desc_size < 0 || img_h > 65535 || img_w > 65535)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  DescGrid g;
  double rect[4];
  if (!feature_grid(img_w, img_h, x_axis, y_axis, desc_step, rect, &g.nx, &g.ny))
    return fail(ctx, PA_ERR_INVALID, "degenerate grid axes or step");
  // patch_scale = (2 * desc_size + 1) / (float)PATCH_SIZE (partdetect_aux.cpp:88); a
  // window wider than the patch samples the image smoothed once with sigma =
  // patch_scale (:92-98)
  const double patch_scale = (2 * desc_size + 1) / (float)21;
  const bool smooth = patch_scale > 1.0;
  if (smooth && (img_h < 5 || img_w < 5))
    return fail(ctx, PA_ERR_INVALID, "the smoothing filter needs images of at least 5 x 5");
  IirCoefs cf;
  if (smooth) smooth_coefficients((float)patch_scale, cf.c);
  g.min_x = rect[0];
  g.min_y = rect[2];
  g.step = desc_step;
  g.ax0 = x_axis[0];
  g.ax1 = x_axis[1];
  g.ay0 = y_axis[0];
  g.ay1 = y_axis[1];
  desc_bounds(g, img_w, img_h, desc_size, roi);
  g.mask = nullptr;
  g.mask_w = img_w;
  g.mask_h = img_h;
  g.mask_ox = g.mask_oy = 0;
  g.v0x = (float)(patch_scale * x_axis[0]);
  g.v0y = (float)(patch_scale * y_axis[0]);
  g.v1x = (float)(patch_scale * x_axis[1]);
  g.v1y = (float)(patch_scale * y_axis[1]);
  DescTables tabs;
  patch_tables(tabs);
  DeviceGuard dg(ctx->device);
  const size_t npx = (size_t)img_h * img_w, ncell = (size_t)g.nx * g.ny;
  float *sm_tmp = nullptr, *sm_out = nullptr;
  auto plan = [&](Builder &b, const DescTables **t, const float **din, float **dout,
                  uint8_t **vout) {
    *t = b.param(&tabs, 1);
    *din = mem == PA_MEM_HOST ? b.scratch<float>(npx) : image;
    if (detection_mask) g.mask = mem == PA_MEM_HOST ? b.scratch<float>(npx) : detection_mask;
    *dout = mem == PA_MEM_HOST ? b.scratch<float>(ncell * 96) : cells;
    *vout = mem == PA_MEM_HOST ? b.scratch<uint8_t>(ncell) : valid;
    sm_tmp = smooth ? b.scratch<float>(npx) : nullptr;
    sm_out = smooth ? b.scratch<float>(npx) : nullptr;
  };
  Builder b1;
  const DescTables *t = nullptr;
  const float *din = nullptr;
  float *dout = nullptr;
  uint8_t *vout = nullptr;
  plan(b1, &t, &din, &dout, &vout);
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  b.base = ctx->arena;
  plan(b, &t, &din, &dout, &vout);
  if ((st = upload_blob(ctx, b))) return st;
  if (mem == PA_MEM_HOST) {
    if ((st = copy_in(ctx, (void *)din, image, npx * sizeof(float), mem))) return st;
    if (detection_mask &&
        (st = copy_in(ctx, (void *)g.mask, detection_mask, npx * sizeof(float), mem)))
      return st;
  }
  if (smooth) {
    PA_LAUNCH_N("smooth", 2, launch_smooth(din, sm_tmp, sm_out, img_h, img_w, cf, ctx->stream));
    din = sm_out;
  }
  PA_LAUNCH("shape_grid", launch_shape_grid(din, img_h, img_w, g, t, dout, vout, ctx->stream));
  if (mem == PA_MEM_HOST) {
    PA_CK(cudaMemcpyAsync(cells, dout, ncell * 96 * sizeof(float), cudaMemcpyDeviceToHost,
                          ctx->stream));
    PA_CK(cudaMemcpyAsync(valid, vout, ncell, cudaMemcpyDeviceToHost, ctx->stream));
  }
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

namespace {

// partdetect_dense at scale index si (partdetect_test.cpp:116-237); writes the
// log unaries of scale si into log_unary [n_cls][S][R][img_h][img_w].
pa_status partdetect_scale(pa_ctx *ctx, const pa_exp_param *ep, int si, const float *image,
                           int img_h, int img_w, int flip, const pa_classifier *const *cls,
                           int n_cls, const pa_part_window *windows, const pa_abc_param *abc,
                           const float *detection_mask, float *log_unary, int mem) {
  const int R = ep->num_rotation_steps, S = n_scales(ep);
  const double scale = scale_from_index(ep, si);
  const double desc_step = scale * abc->desc_step;
  const int desc_size = (int)std::floor(scale * abc->desc_size + 0.5);  // boost_math::round
  double max_part_diag = 0;
  std::vector<int> gx(n_cls), gy(n_cls);
  for (int c = 0; c < n_cls; ++c) {
    if (!cls[c]) return fail(ctx, PA_ERR_INVALID, "classifier %d is NULL", c);
    const pa_part_window &pw = windows[c];
    if (pw.window_size_x < 0 || pw.window_size_y < 0)
      return fail(ctx, PA_ERR_INVALID, "classifier %d: negative window size", c);
    const double d = std::sqrt((double)pw.window_size_x * pw.window_size_x +
                               (double)pw.window_size_y * pw.window_size_y);
    if (d > max_part_diag) max_part_diag = d;
    // get_window_feature_counts, partdetect_aux.cpp:245-250
    gx[c] = pw.window_size_x / abc->desc_step + 1;
    gy[c] = pw.window_size_y / abc->desc_step + 1;
    if ((int64_t)gx[c] * gy[c] * 96 != cls[c]->dim)
      return fail(ctx, PA_ERR_INVALID, "classifier %d has dim %d, its window needs %d x %d x 96",
                  c, cls[c]->dim, gx[c], gy[c]);
  }
  int border = (int)std::ceil(desc_size + 0.5 * scale * max_part_diag);
  if (!(border < img_w && border < img_h)) border = std::min(img_w, img_h) - 1;  // add_image_border2
  const int eh = img_h + 2 * border, ew = img_w + 2 * border;
  double window_step = abc->window_desc_step_ratio * desc_step;
  if (window_step < 1) window_step = 1;
  const double grid_step = desc_step / window_step;
  // cells window_step apart never share a pixel of the TM_DIRECT map when
  // window_step > sqrt 2; closer grids keep the reference's last writer per
  // pixel in a scratch (k_unary_direct_gather)
  const bool ordered = !(window_step * window_step > 2.0);
  // the rotated grids (partdetect_test.cpp:171-185)
  struct Rot {
    double ax[2], ay[2], rect[4];
    int nx, ny;
  };
  std::vector<Rot> rots(R);
  for (int r = 0; r < R; ++r) {
    const double rotation = rot_from_index(ep, r) * (M_PI / 180.0);
    Rot &q = rots[r];
    q.ax[0] = std::cos(rotation);
    q.ax[1] = std::sin(rotation);
    q.ay[0] = -std::sin(rotation);
    q.ay[1] = std::cos(rotation);
    if (flip) {
      q.ax[0] = -q.ax[0];
      q.ax[1] = -q.ax[1];
    }
    if (!feature_grid(ew, eh, q.ax, q.ay, window_step, q.rect, &q.nx, &q.ny))
      return fail(ctx, PA_ERR_INVALID, "rotation %d: degenerate grid", r);
  }
  const double patch_scale = (2 * desc_size + 1) / (float)21;
  const bool smooth = patch_scale > 1.0;
  IirCoefs cf;
  if (smooth) smooth_coefficients((float)patch_scale, cf.c);
  DescTables tabs;
  patch_tables(tabs);
  // classifier groups by window shape (one window gather + one score launch each)
  std::vector<int> order(n_cls);
  for (int c = 0; c < n_cls; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return gx[a] != gx[b] ? gx[a] < gx[b] : gy[a] < gy[b];
  });
  std::vector<std::pair<int, int>> groups;  // [first, end) in `order`
  for (int k = 0; k < n_cls; ++k)
    if (k == 0 || gx[order[k]] != gx[order[k - 1]] || gy[order[k]] != gy[order[k - 1]])
      groups.push_back({k, k + 1});
    else
      groups.back().second = k + 1;
  std::vector<const pa_classifier *> cls_sorted(n_cls);
  for (int k = 0; k < n_cls; ++k) cls_sorted[k] = cls[order[k]];
  size_t max_cells = 0, max_dense = 0, total_scores = 0;
  std::vector<size_t> score_off(R);
  for (int r = 0; r < R; ++r) {
    const size_t G = (size_t)rots[r].nx * rots[r].ny;
    max_cells = std::max(max_cells, G);
    for (auto &g : groups)
      max_dense = std::max(max_dense, G * (size_t)gx[order[g.first]] * gy[order[g.first]] * 96);
    score_off[r] = total_scores;
    total_scores += G * n_cls;
  }
  const size_t npx = (size_t)img_h * img_w, nepx = (size_t)eh * ew;
  DeviceGuard dg(ctx->device);
  struct Dev {
    const DescTables *tabs;
    StumpPart *sp;
    const float *img, *mask;
    float *ext, *sm_tmp, *sm_out, *cells, *dense, *scores, *out;
    uint8_t *valid, *ok;
    int4 *bbox;
    const float **grid_ptrs;
    UnaryMap *maps;
    int *order;
  } d{};
  std::vector<const float *> grid_ptrs((size_t)R * n_cls);
  auto plan = [&](Builder &b) {
    d.tabs = b.param(&tabs, 1);
    d.sp = plan_stumps(b, cls_sorted.data(), n_cls);
    d.img = mem == PA_MEM_HOST ? b.scratch<float>(npx) : image;
    // this scale's detection mask [img_h][img_w]
    d.mask = !detection_mask ? nullptr
             : mem == PA_MEM_HOST ? b.scratch<float>(npx)
                                  : detection_mask + (size_t)si * npx;
    d.ext = b.scratch<float>(nepx);
    d.sm_tmp = smooth ? b.scratch<float>(nepx) : nullptr;
    d.sm_out = smooth ? b.scratch<float>(nepx) : nullptr;
    d.cells = b.scratch<float>(max_cells * 96);
    d.valid = b.scratch<uint8_t>(max_cells);
    d.dense = b.scratch<float>(max_dense);
    d.ok = b.scratch<uint8_t>(max_cells);
    d.scores = b.scratch<float>(total_scores);
    d.bbox = b.scratch<int4>((size_t)R * n_cls);
    for (int r = 0; r < R; ++r)
      for (int k = 0; k < n_cls; ++k)
        grid_ptrs[(size_t)r * n_cls + k] =
            b.dry ? nullptr : d.scores + score_off[r] + (size_t)k * rots[r].nx * rots[r].ny;
    d.grid_ptrs = b.param(grid_ptrs.data(), grid_ptrs.size());
    d.maps = b.scratch<UnaryMap>((size_t)R * n_cls + 1);  // + 1: the 16-byte copy tail
    // one rotation's last writers, reused by the next (stream order)
    d.order = ordered ? b.scratch<int>((size_t)n_cls * npx) : nullptr;
    // host memory: this scale's [n_cls][R][img_h][img_w] block, copied out below
    d.out = mem == PA_MEM_HOST ? b.scratch<float>((size_t)n_cls * R * npx) : log_unary;
  };
  const size_t cstride = (mem == PA_MEM_HOST ? (size_t)R : (size_t)S * R) * npx;  // per classifier
  const size_t sofs = mem == PA_MEM_HOST ? 0 : (size_t)si * R * npx;
  Builder b1;
  plan(b1);
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  b.base = ctx->arena;
  plan(b);
  if ((st = upload_blob(ctx, b))) return st;
  cudaStream_t s = ctx->stream;
  if (mem == PA_MEM_HOST) {
    if ((st = copy_in(ctx, (void *)d.img, image, npx * sizeof(float), mem))) return st;
    if (d.mask && (st = copy_in(ctx, (void *)d.mask, detection_mask + (size_t)si * npx,
                                npx * sizeof(float), mem)))
      return st;
  }
  PA_LAUNCH_N("border", border > 0 ? 2 : 1, launch_mirror_border(d.img, img_h, img_w, border, d.ext, s));
  const float *src = d.ext;
  if (smooth) {
    PA_LAUNCH_N("smooth", 2, launch_smooth(d.ext, d.sm_tmp, d.sm_out, eh, ew, cf, s));
    src = d.sm_out;
  }
  const std::vector<char> ff = fast_flags(cls_sorted.data(), n_cls);
  const std::vector<int> ns = stump_counts(cls_sorted.data(), n_cls);
  for (int r = 0; r < R; ++r) {
    const Rot &q = rots[r];
    DescGrid g;
    g.min_x = q.rect[0];
    g.min_y = q.rect[2];
    g.step = window_step;
    g.ax0 = q.ax[0];
    g.ax1 = q.ax[1];
    g.ay0 = q.ay[0];
    g.ay1 = q.ay[1];
    desc_bounds(g, ew, eh, desc_size, nullptr);
    // the mask sits in a zero array the size of the bordered image, at
    // (border, border) (partdetect_test.cpp:135-146)
    g.mask = d.mask;
    g.mask_w = img_w;
    g.mask_h = img_h;
    g.mask_ox = g.mask_oy = border;
    g.v0x = (float)(patch_scale * q.ax[0]);
    g.v0y = (float)(patch_scale * q.ay[0]);
    g.v1x = (float)(patch_scale * q.ax[1]);
    g.v1y = (float)(patch_scale * q.ay[1]);
    g.nx = q.nx;
    g.ny = q.ny;
    PA_LAUNCH("shape_grid", launch_shape_grid(src, eh, ew, g, d.tabs, d.cells, d.valid, s));
    const int64_t G = (int64_t)q.nx * q.ny;
    for (auto &grp : groups) {
      const int c0 = order[grp.first], n = grp.second - grp.first;
      const int D = gx[c0] * gy[c0] * 96;
      PA_LAUNCH("window_gather", launch_window_gather(d.cells, d.valid, 1, q.ny, q.nx, 96, gx[c0],
                                                      gy[c0], grid_step, d.dense, d.ok, s));
      float *sc = d.scores + score_off[r] + (size_t)grp.first * G;
      PA_LAUNCH("score_grids",
                launch_score_grids(d.sp + grp.first, (const bool *)ff.data() + grp.first,
                                   ns.data() + grp.first, n, d.dense, nullptr, false, G, 1, D, 1,
                                   sc, s));
      PA_LAUNCH("mask_no_class", launch_mask_no_class(sc, d.ok, n, G, s));
    }
    PA_LAUNCH("grid_bbox", launch_grid_bbox(d.grid_ptrs + (size_t)r * n_cls, n_cls, q.ny, q.nx,
                                            d.bbox + (size_t)r * n_cls, s));
  }
  std::vector<int4> bbox((size_t)R * n_cls);
  PA_CK(cudaMemcpyAsync(bbox.data(), d.bbox, bbox.size() * sizeof(int4), cudaMemcpyDeviceToHost, s));
  if ((st = sync_ctx(ctx))) return st;
  // computeScoreGrid's transforms (partdetect_test.cpp:379-403), squeezeScoreGrid
  // (:407-449) and Tig = (Ti_ei Ti2)(T2g Tg4) (:205-213, 272-283), host double
  std::vector<UnaryMap> maps((size_t)R * n_cls);
  for (int r = 0; r < R; ++r) {
    const Rot &q = rots[r];
    const double T32[9] = {1, 0, -q.rect[0], 0, 1, -q.rect[2], 0, 0, 1};
    double T23[9];
    hc_inverse(T32, T23);
    const double Ti2[9] = {q.ax[0], q.ay[0], 0, q.ax[1], q.ay[1], 0, 0, 0, 1};
    const double Tie[9] = {1, 0, (double)-border, 0, 1, (double)-border, 0, 0, 1};
    double Ti2e[9];
    prod3(Tie, Ti2, Ti2e);
    for (int k = 0; k < n_cls; ++k) {
      const int c = order[k];
      const pa_part_window &pw = windows[c];
      double T3g[9] = {window_step, 0, 0, 0, window_step, 0, 0, 0, 1};
      T3g[2] = scale * pw.pos_offset_x;
      T3g[5] = scale * pw.pos_offset_y;
      double T2g[9], Tig[9];
      prod3(T23, T3g, T2g);
      const int4 bb = bbox[(size_t)r * n_cls + k];
      int ox = 0, oy = 0;
      if (bb.z > bb.x && bb.w > bb.y) {  // maxx > minx && maxy > miny
        const double Tg4[9] = {1, 0, (double)bb.x, 0, 1, (double)bb.y, 0, 0, 1};
        double M[9];
        prod3(T2g, Tg4, M);
        std::memcpy(T2g, M, sizeof M);
        ox = bb.x;
        oy = bb.y;
      }
      prod3(Ti2e, T2g, Tig);
      UnaryMap &m = maps[(size_t)r * n_cls + k];
      std::memset(&m, 0, sizeof m);
      m.grid = grid_ptrs[(size_t)r * n_cls + k];
      m.out = d.out + c * cstride + sofs + (size_t)r * npx;
      for (int t = 0; t < 6; ++t) m.T31[t] = Tig[t];
      m.ox = ox;
      m.oy = oy;
      m.order = ordered ? d.order + (size_t)k * npx : nullptr;
    }
  }
  if ((st = upload_to(ctx, d.maps, maps.data(), maps.size() * sizeof(UnaryMap)))) return st;
  for (int r = 0; r < R; ++r)
    PA_LAUNCH_N("unary_maps", ordered ? 3 : 2,
                launch_unary_maps(d.maps + (size_t)r * n_cls, n_cls, rots[r].ny, rots[r].nx,
                                  img_h, img_w, 1, 0, ordered, s));
  if (mem == PA_MEM_HOST)
    PA_CK(cudaMemcpy2DAsync(log_unary + (size_t)si * R * npx, (size_t)S * R * npx * sizeof(float),
                            d.out, (size_t)R * npx * sizeof(float), (size_t)R * npx * sizeof(float),
                            (size_t)n_cls, cudaMemcpyDeviceToHost, s));
  return sync_ctx(ctx);
}

}  // namespace

pa_status pa_partdetect(pa_ctx *ctx, const pa_exp_param *ep, const float *image, int img_h,
                        int img_w, int flip, const pa_classifier *const *cls, int n_cls,
                        const pa_part_window *windows, const pa_abc_param *abc,
                        float *log_unary, int mem) {
  return pa_partdetect_masked(ctx, ep, image, img_h, img_w, flip, cls, n_cls, windows, abc,
                              nullptr, log_unary, mem);
}

pa_status pa_partdetect_masked(pa_ctx *ctx, const pa_exp_param *ep, const float *image,
                               int img_h, int img_w, int flip, const pa_classifier *const *cls,
                               int n_cls, const pa_part_window *windows,
                               const pa_abc_param *abc, const float *detection_mask,
                               float *log_unary, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!exp_ok(ep)) return fail(ctx, PA_ERR_INVALID, "invalid experiment parameters");
  if (!image || !log_unary || !windows || !abc || img_h < 5 || img_w < 5 || img_h > 16384 ||
      img_w > 16384 || abc->desc_step < 1 || abc->desc_size < 0 ||
      !(abc->window_desc_step_ratio > 0 && abc->window_desc_step_ratio <= 1))
    return fail(ctx, PA_ERR_INVALID, "invalid sizes, parameters or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  if (!cls || n_cls < 1) return fail(ctx, PA_ERR_INVALID, "no classifiers");
  // the scale loop of partdetect_dense (partdetect_test.cpp:116): every scale
  // its own descriptor step and size, border, grids and windows
  for (int si = 0; si < n_scales(ep); ++si)
    if (pa_status st = partdetect_scale(ctx, ep, si, image, img_h, img_w, flip, cls, n_cls,
                                        windows, abc, detection_mask, log_unary, mem))
      return st;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_score_grids_window(pa_ctx *ctx, const pa_classifier *const *cls, int n_parts,
                                const float *cells, const uint8_t *valid, int n_fields, int ny,
                                int nx, int dc, int gx, int gy, double grid_step, int normalize,
                                float *scores, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!cells || !valid || !scores || n_fields < 1 || ny < 1 || nx < 1 || dc < 1 || gx < 1 ||
      gy < 1 || !(grid_step > 0))
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  const int D = gx * gy * dc;
  pa_status st = check_classifiers(ctx, cls, n_parts, D);
  if (st) return st;
  DeviceGuard dg(ctx->device);
  const int64_t G = (int64_t)ny * nx;
  const size_t ncell = (size_t)n_fields * G * dc, nval = (size_t)n_fields * G;
  const size_t ndense = (size_t)n_fields * G * D, dout = (size_t)n_parts * n_fields * G;
  Builder b1;
  plan_stumps(b1, cls, n_parts);
  b1.scratch<float>(ndense);
  b1.scratch<uint8_t>(nval);
  if (mem == PA_MEM_HOST) {
    b1.scratch<float>(ncell);
    b1.scratch<uint8_t>(nval);
    b1.scratch<float>(dout);
  }
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  st = ensure_arena(ctx, b1.total());
  if (st) return st;
  b.base = ctx->arena;
  StumpPart *sp = plan_stumps(b, cls, n_parts);
  float *dense = b.scratch<float>(ndense);
  uint8_t *ok = b.scratch<uint8_t>(nval);
  const float *d_cells = cells;
  const uint8_t *d_valid = valid;
  float *d_out = scores;
  if (mem == PA_MEM_HOST) {
    d_cells = b.scratch<float>(ncell);
    d_valid = b.scratch<uint8_t>(nval);
    d_out = b.scratch<float>(dout);
  }
  st = upload_blob(ctx, b);
  if (st) return st;
  if (mem == PA_MEM_HOST) {
    if ((st = copy_in(ctx, (void *)d_cells, cells, ncell * sizeof(float), mem))) return st;
    if ((st = copy_in(ctx, (void *)d_valid, valid, nval, mem))) return st;
  }
  cudaStream_t s = ctx->stream;
  PA_LAUNCH("window_gather", launch_window_gather(d_cells, d_valid, n_fields, ny, nx, dc, gx, gy, grid_step, dense,
                                 ok, s));
  const std::vector<char> ff = fast_flags(cls, n_parts);
  const std::vector<int> ns = stump_counts(cls, n_parts);
  PA_LAUNCH("score_grids", launch_score_grids(sp, (const bool *)ff.data(), ns.data(), n_parts, dense, nullptr, false, G,
                                              n_fields, D, normalize, d_out, s));
  PA_LAUNCH("mask_no_class", launch_mask_no_class(d_out, ok, n_parts, (int64_t)n_fields * G, s));
  if (mem == PA_MEM_HOST)
    PA_CK(cudaMemcpyAsync(scores, d_out, dout * sizeof(float), cudaMemcpyDeviceToHost, s));
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_maps(pa_ctx *ctx, const float *scores, int n_parts, int R, int ny, int nx,
                        const double *Tig, int tig_shared, int interpolate, int H, int W,
                        float *log_unary, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!scores || !Tig || !log_unary || n_parts < 1 || R < 1 || ny < 1 || nx < 1 || H < 1 || W < 1)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  DeviceGuard dg(ctx->device);
  const size_t nin = (size_t)n_parts * R * ny * nx, nout = (size_t)n_parts * R * H * W;
  pa_exp_param e;
  pa_exp_param_default(&e);
  e.num_rotation_steps = R;
  std::vector<int> upright(n_parts, 0);
  std::vector<std::vector<float *>> outs(1, std::vector<float *>(n_parts, nullptr));
  UnaryMap *maps = nullptr;
  Builder b1;
  const float *d_in = scores;
  float *d_out = log_unary;
  if (mem == PA_MEM_HOST) {
    b1.scratch<float>(nin);
    b1.scratch<float>(nout);
  }
  int usep = 0;
  pa_status st = plan_unary(ctx, b1, Tig, tig_shared, 1, n_parts, R, ny, nx, H, W, !interpolate,
                            d_in, R, outs, upright, 0, 0.f, nullptr, &e, &maps, 0, &usep);
  if (st) return st;
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  if ((st = ensure_arena(ctx, b1.total()))) return st;
  b.base = ctx->arena;
  if (mem == PA_MEM_HOST) {
    d_in = b.scratch<float>(nin);
    d_out = b.scratch<float>(nout);
  }
  for (int p = 0; p < n_parts; ++p) outs[0][p] = d_out + (size_t)p * R * H * W;
  st = plan_unary(ctx, b, Tig, tig_shared, 1, n_parts, R, ny, nx, H, W, !interpolate, d_in, R,
                  outs, upright, 0, 0.f, nullptr, &e, &maps, 0, &usep);
  if (st) return st;
  if ((st = upload_blob(ctx, b))) return st;
  if (mem == PA_MEM_HOST)
    if ((st = copy_in(ctx, (void *)d_in, scores, nin * sizeof(float), mem))) return st;
  PA_LAUNCH_N("unary_maps", unary_launches(!interpolate, usep),
              launch_unary_maps(maps, n_parts * R, ny, nx, H, W, !interpolate,
                                usep & kUnarySeparable, usep & kUnaryOrdered, ctx->stream));
  if (mem == PA_MEM_HOST)
    PA_CK(cudaMemcpyAsync(log_unary, d_out, nout * sizeof(float), cudaMemcpyDeviceToHost,
                          ctx->stream));
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

namespace {

// pa_ps_infer with the log unaries in unary_mem and the outputs in mem.
pa_status ps_infer_impl(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                        int is_sparse, const float *log_unary, int unary_mem, int H, int W,
                        const pa_ps_outputs *out, int mem) {
  PsPlan pl;
  pl.tc_mode = ctx->msg_math == PA_MSG_BF16_TENSOR;
  pl.sparse_up = is_sparse != 0;
  pa_status st = build_sched(ctx, tree, pl.sc);
  if (st) return st;
  // computeRootPosteriorRot runs one independent pass per scale
  // (objectdetect_findrot.cpp:503-678): the scales are the entries of a batch
  const int S = n_scales(ep);
  std::vector<std::vector<Joint>> joints(S);
  if ((st = load_joints(ctx, tree, flip, joints[0]))) return st;
  for (int sc = 1; sc < S; ++sc) joints[sc] = joints[0];
  const int P = pl.sc.P, R = ep->num_rotation_steps;
  pl.B = S;
  pl.P = P;
  pl.R = R;
  pl.H = H;
  pl.W = W;
  pl.N = (int64_t)R * H * W;
  const int64_t HW = (int64_t)H * W;
  // best_part_hyp holds the last scale's maxima (computePartMarginals clears it
  // per scale, :254-258); getMaxStates reads scale 0 (:78)
  const int hyp_scale = ep->use_pairwise ? S - 1 : 0;
  if (S > 1) {
    for (int sc = 0; sc < S; ++sc) pl.img_scale.push_back(sc);
    pl.out_pstride = (int64_t)S * pl.N;
    pl.hyp_img = hyp_scale;
    pl.root_joint = true;
  }
  std::vector<pa_ps_outputs> outs(S);
  for (int sc = 0; sc < S; ++sc) {
    pa_ps_outputs &o = outs[sc];
    o = *out;
    if (S == 1) break;
    o.log_marg = out->log_marg ? out->log_marg + sc * pl.N : nullptr;
    o.root_post = out->root_post ? out->root_post + sc * HW : nullptr;
    o.log_z = out->log_z ? out->log_z + (size_t)sc * P : nullptr;
    o.msg_max = out->msg_max ? out->msg_max + (size_t)sc * 2 * std::max(1, P - 1) : nullptr;
    if (sc != hyp_scale) o.best = nullptr, o.part_hyps = nullptr, o.n_part_hyps = nullptr;
    if (sc != 0) o.root_hyps = nullptr, o.n_root_hyps = nullptr;
  }
  DeviceGuard dg(ctx->device);
  std::vector<float *> marg_out(S, nullptr), rp_out(S, nullptr);
  if (mem == PA_MEM_DEVICE)
    for (int sc = 0; sc < S; ++sc) {
      marg_out[sc] = outs[sc].log_marg;
      rp_out[sc] = outs[sc].root_post;
    }
  std::vector<int> masked((size_t)P * R, 0);
  for (int p = 0; p < P; ++p)
    if (pl.sc.upright[p])
      for (int r = 0; r < R; ++r) masked[(size_t)p * R + r] = !(std::fabs(rot_from_index(ep, r)) < 15.0);
  auto plan = [&](Builder &b, PsPlan &p2, int **masked_dev, const float **unary_dev) {
    *masked_dev = b.param(masked.data(), masked.size());
    *unary_dev = (unary_mem == PA_MEM_HOST) ? b.scratch<float>((size_t)P * S * pl.N) : log_unary;
    std::vector<float *> rp = rp_out;
    if (S > 1 && !rp[0]) {  // the scales' root posteriors form one [S][H][W] grid
      float *g = b.scratch<float>((size_t)S * HW);
      for (int sc = 0; sc < S; ++sc) rp[sc] = g + sc * HW;
    }
    plan_ps(b, p2, ep, joints, marg_out.data(), rp.data());
    plan_marg_ptrs(b, p2);
    plan_localmax(b, p2, ep, outs.data());
  };
  Builder b1;
  PsPlan pl1 = pl;
  int *mk = nullptr;
  const float *ud = nullptr;
  plan(b1, pl1, &mk, &ud);
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  if ((st = ensure_arena(ctx, b1.total()))) return st;
  b.base = ctx->arena;
  PsPlan pl2 = pl;
  plan(b, pl2, &mk, &ud);
  if ((st = upload_blob(ctx, b))) return st;
  if (unary_mem == PA_MEM_HOST)
    if ((st = copy_in(ctx, (void *)ud, log_unary, (size_t)P * S * pl.N * sizeof(float), unary_mem)))
      return st;
  if ((st = init_slots(ctx, pl2))) return st;
  cudaStream_t s = ctx->stream;
  const int strip = (int)(ep->strip_border_detections * W);
  for (int sc = 0; sc < S; ++sc)
    for (int p = 0; p < P; ++p) {
      float *dst = ep->use_pairwise ? pl2.im[sc].U[p] : pl2.im[sc].MARG[p];
      PA_LAUNCH("prepare_unary",
                launch_prepare_unary(ud + ((size_t)p * S + sc) * pl.N, dst,
                                     pl2.sc.upright[p] ? mk + (size_t)p * R : nullptr,
                                     p == pl2.sc.root ? strip : 0, R, H, W,
                                     pl2.umax + (size_t)sc * P + p, s));
    }
  if ((st = run_ps(ctx, ep, pl2))) return st;
  return finish_ps(ctx, ep, pl2, outs.data(), mem);
}

}  // namespace

pa_status pa_ps_infer(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                      int is_sparse, const float *log_unary, int H, int W,
                      const pa_ps_outputs *out, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!exp_ok(ep)) return fail(ctx, PA_ERR_INVALID, "invalid experiment parameters");
  if (!tree || !log_unary || !out || H < 1 || W < 1 || H > 32767 || W > 32767)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  return ps_infer_impl(ctx, ep, tree, flip, is_sparse, log_unary, mem, H, W, out, mem);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_rot_joint_marginal(pa_ctx *ctx, const pa_exp_param *ep, const float *child,
                                float *parent, int R, int H, int W, const double *offset_c,
                                const double *offset_p, const double *C, double rot_mean,
                                double rot_sigma, double scale, int is_sparse, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!ep || !child || !parent || !offset_c || !offset_p || !C || H < 1 || W < 1 ||
      H > 32767 || W > 32767 || R != ep->num_rotation_steps || !exp_ok(ep))
    return fail(ctx, PA_ERR_INVALID, "invalid sizes, parameters or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  if (!cov_ok(C)) return fail(ctx, PA_ERR_INVALID, "covariance must be symmetric positive definite");
  DeviceGuard dg(ctx->device);
  const int64_t N = (int64_t)R * H * W;
  MsgParams mp;
  msg_params(ep, scale, offset_c, offset_p, C, rot_mean, rot_sigma, H, W, is_sparse != 0, mp);
  int4 *sdesc = nullptr;
  auto plan = [&](Builder &b, MsgDesc **md, int16_t **tables, double **shifts, int **slot,
                  int **err, const float **din, float **dout, float **e2) {
    MsgDesc d;
    std::memset(&d, 0, sizeof d);
    *tables = b.scratch<int16_t>((size_t)2 * R * (W + H));
    sdesc = b.scratch<int4>((size_t)4 * R);
    d.sdesc = sdesc;
    *slot = b.scratch<int>(1);
    *err = b.scratch<int>(1);
    *e2 = b.scratch<float>(N);
    if (mp.full) {
      d.full = 1;
      d.oh = mp.oh;
      d.ow = mp.ow;
      d.g0 = b.scratch<float>((size_t)R * mp.oh * mp.ow);
      d.g1 = b.scratch<float>((size_t)R * mp.oh * mp.ow);
      for (int q = 0; q < 6; ++q) {
        d.tf[q] = mp.tf[q];
        d.tb[q] = mp.tb[q];
        d.td[q] = mp.td[q];
      }
      d.sparse = mp.sparse ? 1 : 0;
    }
    *din = (mem == PA_MEM_HOST) ? b.scratch<float>(N) : child;
    *dout = (mem == PA_MEM_HOST) ? b.scratch<float>(N) : parent;
    d.in = *din;
    d.in_max = *slot;
    d.e2 = *e2;
    d.tx_in = *tables;
    d.ty_in = b.dry ? nullptr : *tables + (size_t)R * W;
    d.tx_out = b.dry ? nullptr : *tables + (size_t)R * (W + H);
    d.ty_out = b.dry ? nullptr : *tables + (size_t)R * (W + H) + (size_t)R * W;
    d.rtaps = mp.rtaps.empty() ? nullptr : b.param(mp.rtaps.data(), mp.rtaps.size());
    d.xtaps = b.param(mp.xtaps.data(), mp.xtaps.size());
    d.ytaps = b.param(mp.ytaps.data(), mp.ytaps.size());
    d.kidx = mp.kidx;
    d.rlen = mp.rlen;
    d.xlen = mp.xlen;
    d.ylen = mp.ylen;
    d.mode = EPI_STORE;
    d.dst0 = *dout;
    *shifts = b.param(mp.shifts.data(), mp.shifts.size());
    *md = b.param(&d, 1);
  };
  MsgDesc *md;
  int16_t *tables;
  double *shifts;
  int *slot, *err;
  const float *din;
  float *dout, *e2;
  Builder b1;
  plan(b1, &md, &tables, &shifts, &slot, &err, &din, &dout, &e2);
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  b.base = ctx->arena;
  plan(b, &md, &tables, &shifts, &slot, &err, &din, &dout, &e2);
  if ((st = upload_blob(ctx, b))) return st;
  cudaStream_t s = ctx->stream;
  if (mem == PA_MEM_HOST)
    if ((st = copy_in(ctx, (void *)din, child, N * sizeof(float), mem))) return st;
  PA_LAUNCH("fill", launch_fill_int(slot, kFkeyNegInf, 1, s));
  PA_CK(cudaMemsetAsync(err, 0, sizeof(int), s));
  PA_LAUNCH("map_max", launch_map_max(din, N, slot, s));
  PA_LAUNCH_N("shift_tables", 2, launch_shift_tables(shifts, 1, R, H, W, tables, sdesc, s));
  PA_LAUNCH("msg_rows", launch_msg_rows(md, 1, R, H, W, (mp.xlen - 1) / 2, err, s));
  if (mp.full)
    PA_LAUNCH_N("msg_full", 7, launch_msg_full(md, 1, R, H, W, mp.oh, mp.ow, (mp.xlen - 1) / 2,
                                               (mp.ylen - 1) / 2, err, s));
  else
    PA_LAUNCH("msg_cols", launch_msg_cols(md, 1, R, H, W, (mp.ylen - 1) / 2, err, s));
  if (mem == PA_MEM_HOST)
    PA_CK(cudaMemcpyAsync(parent, dout, N * sizeof(float), cudaMemcpyDeviceToHost, s));
  int errflag = 0;
  PA_CK(cudaMemcpyAsync(&errflag, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (pa_status ss = sync_ctx(ctx)) return ss;
  if (errflag & 1)
    return fail(ctx, PA_ERR_NUMERIC, "exp() overflowed in the message (the reference asserts here)");
  if (errflag) return fail(ctx, PA_ERR_UNSUPPORTED, "message kernel rejected its input (code %d)", errflag);
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_gemm_bf16(pa_ctx *ctx, const void *A, int64_t lda, const void *B, int64_t ldb,
                       float *C, int64_t ldc, int M, int N, int K, int band) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!A || !B || !C || M < 1 || N < 1 || K < 1 || lda < K || ldb < K || ldc < N || lda % 8 ||
      ldb % 8 || ((uintptr_t)A & 15) || ((uintptr_t)B & 15))
    return fail(ctx, PA_ERR_INVALID, "invalid GEMM operands");
  DeviceGuard dg(ctx->device);
  Builder b1;
  int *err1 = b1.scratch<int>(1);
  (void)err1;
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  int *err = reinterpret_cast<int *>(ctx->arena);
  cudaStream_t s = ctx->stream;
  PA_CK(cudaMemsetAsync(err, 0, sizeof(int), s));
  GemmArgs g{};
  g.C = C;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ldc = ldc;
  g.band = band < 0 ? -1 : band;
  PA_LAUNCH("gemm_bf16", launch_tc_gemm(A, lda, M, K, B, ldb, N, K, g, 1, err, s));
  int flag = 0;
  PA_CK(cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (pa_status ss = sync_ctx(ctx)) return ss;
  if (flag) return fail(ctx, PA_ERR_CUDA, "GEMM pipeline wait timed out (flag %d)", flag);
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_find_obj(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                      const pa_classifier *const *cls, int n_cls, const float *desc, int ny,
                      int nx, int dim, const double *Tig, int tig_shared, int H, int W,
                      float *scores_out, const pa_ps_outputs *out, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  return find_obj_impl(ctx, ep, 1, tree, flip, cls, n_cls, desc, ny, nx, dim, Tig, tig_shared, H,
                       W, scores_out, out, mem);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_find_obj_batch(pa_ctx *ctx, const pa_exp_param *ep, int n_images,
                            const pa_tree *trees, int flip, const pa_classifier *const *cls,
                            int n_cls, const float *desc, int ny, int nx, int dim,
                            const double *Tig, int tig_shared, int H, int W, float *scores_out,
                            const pa_ps_outputs *out, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  return find_obj_impl(ctx, ep, n_images, trees, flip, cls, n_cls, desc, ny, nx, dim, Tig,
                       tig_shared, H, W, scores_out, out, mem);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_find_obj_scales(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                             const pa_classifier *const *cls, int n_cls,
                             const pa_scale_fields *fields, int H, int W,
                             const pa_ps_outputs *out, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!ep || !exp_ok(ep)) return fail(ctx, PA_ERR_INVALID, "invalid experiment parameters");
  if (!tree || !cls || !fields || !out || H < 1 || W < 1 || H > 32767 || W > 32767)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  const int S = n_scales(ep), R = ep->num_rotation_steps, P = tree->n_parts;
  if (P < 1 || n_cls < P) return fail(ctx, PA_ERR_INVALID, "fewer classifiers than parts");
  size_t max_scores = 0;
  for (int sc = 0; sc < S; ++sc) {
    const pa_scale_fields &f = fields[sc];
    if (!f.desc || !f.Tig || f.ny < 1 || f.nx < 1 || f.dim < 1)
      return fail(ctx, PA_ERR_INVALID, "scale %d: invalid fields", sc);
    max_scores = std::max(max_scores, (size_t)P * R * f.ny * f.nx);
  }
  DeviceGuard dg(ctx->device);
  // one device block outlives the arena-using calls below: the unaries of
  // every scale, then one scale's scores and unary maps
  const size_t N = (size_t)R * H * W;
  const size_t n_lu = (size_t)P * S * N, n_map = (size_t)P * N;
  const size_t need = (n_lu + n_map + max_scores) * sizeof(float) + 512;
  if (ctx->scales_cap < need) {
    PA_CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->scales_buf) cudaFree(ctx->scales_buf);
    ctx->scales_buf = nullptr;
    ctx->scales_cap = 0;
    if (cudaMalloc(&ctx->scales_buf, need) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, PA_ERR_NOMEM, "device memory exhausted (%zu bytes)", need);
    }
    ctx->scales_cap = need;
  }
  float *lu = reinterpret_cast<float *>(ctx->scales_buf);
  float *maps = lu + n_lu;
  float *scores = reinterpret_cast<float *>(
      (reinterpret_cast<uintptr_t>(maps + n_map) + 255) & ~(uintptr_t)255);
  // per scale: partdetect_dense's score grids with normalised votes, the
  // grid -> image maps, clip + log (objectdetect_findrot.cpp:834-845), into
  // the [P][S][R][H][W] block computeRootPosteriorRot reads
  for (int sc = 0; sc < S; ++sc) {
    const pa_scale_fields &f = fields[sc];
    pa_status st = score_grids_impl(ctx, cls, P, f.desc, mem, R, f.ny, f.nx, f.dim, 1, scores,
                                    PA_MEM_DEVICE);
    if (st) return st;
    if ((st = pa_unary_maps(ctx, scores, P, R, f.ny, f.nx, f.Tig, f.tig_shared, ep->interpolate,
                            H, W, maps, PA_MEM_DEVICE)))
      return st;
    PA_CK(cudaMemcpy2DAsync(lu + (size_t)sc * N, S * N * sizeof(float), maps, N * sizeof(float),
                            N * sizeof(float), (size_t)P, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  // findObjectImageRotJoints passes bIsSparse = true (objectdetect_findrot.cpp:740)
  return ps_infer_impl(ctx, ep, tree, flip, 1, lu, PA_MEM_DEVICE, H, W, out, mem);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_find_obj_multi(pa_ctx *ctx, int n_images, const pa_image *imgs,
                            const pa_classifier *const *cls, int n_cls, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (n_images < 1 || !imgs || !cls || n_cls < 1)
    return fail(ctx, PA_ERR_INVALID, "invalid image list");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  for (int i = 0; i < n_images; ++i) {
    const pa_image &im = imgs[i];
    if (!im.ep || !exp_ok(im.ep) || !im.tree || !im.desc || !im.Tig || !im.out || im.ny < 1 ||
        im.nx < 1 || im.dim < 1 || im.H < 1 || im.W < 1 || im.H > 32767 || im.W > 32767)
      return fail(ctx, PA_ERR_INVALID, "image %d: invalid sizes, parameters or NULL input", i);
    if (n_scales(im.ep) != 1)
      return fail(ctx, PA_ERR_UNSUPPORTED, "image %d: one scale of descriptors per image", i);
  }
  // images that share every size, parameter and transform run as one batch
  auto same = [&](const pa_image &a, const pa_image &b) {
    if (std::memcmp(a.ep, b.ep, sizeof(pa_exp_param)) != 0) return false;
    if (a.flip != b.flip || a.ny != b.ny || a.nx != b.nx || a.dim != b.dim || a.H != b.H ||
        a.W != b.W || !a.tig_shared || !b.tig_shared)
      return false;
    return std::memcmp(a.Tig, b.Tig, 9 * sizeof(double)) == 0 && same_topology(a.tree, b.tree);
  };
  std::vector<int> group(n_images, -1);
  int n_groups = 0;
  for (int i = 0; i < n_images; ++i) {
    if (group[i] >= 0) continue;
    group[i] = n_groups;
    for (int j = i + 1; j < n_images; ++j)
      if (group[j] < 0 && same(imgs[i], imgs[j])) group[j] = n_groups;
    ++n_groups;
  }
  pa_status result = PA_OK;
  if (mem == PA_MEM_DEVICE && n_groups > 1) {
    // Device inputs: the groups run on up to kWorkers worker contexts, each
    // with its own stream and workspace, so that the small grids of several
    // images fill the GPU together.  On each worker the groups are queued
    // back to back: the host plans group g + NW while the GPU computes the
    // worker's previous groups; each group's small results land in one of
    // the worker's pinned slots and are decoded once its stream has passed
    // them, before the slot is reused.
    DeviceGuard dg(ctx->device);
    const int NW = std::min(n_groups, pa_ctx::kWorkers);
    while ((int)ctx->workers.size() < NW) {
      pa_ctx *w = nullptr;
      if (pa_ctx_create(ctx->device, &w) != PA_OK)
        return fail(ctx, PA_ERR_CUDA, "cannot create a worker context");
      ctx->workers.push_back(w);
    }
    while (ctx->ring_done.empty()) {
      cudaEvent_t ev;
      PA_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      ctx->ring_done.push_back(ev);
    }
    // the workers start behind everything queued on the caller's stream
    PA_CK(cudaEventRecord(ctx->ring_done[0], ctx->stream));
    const int nslots = pa_ctx::kLandings;
    struct WorkerState {
      std::vector<PendingImage> pend;
      std::vector<const pa_exp_param *> pend_e;
      int count = 0;
    };
    std::vector<WorkerState> ws(NW);
    for (int w = 0; w < NW; ++w) {
      pa_ctx *wc = ctx->workers[w];
      wc->msg_math = ctx->msg_math;
      wc->timing = ctx->timing;
      while ((int)wc->ring_done.size() < nslots) {
        cudaEvent_t ev;
        PA_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        wc->ring_done.push_back(ev);
      }
      PA_CK(cudaStreamWaitEvent(wc->stream, ctx->ring_done[0], 0));
      ws[w].pend.resize(nslots);
      ws[w].pend_e.assign(nslots, nullptr);
    }
    std::vector<std::vector<pa_ps_outputs>> gouts(n_groups);
    auto drain = [&]() {
      for (int w = 0; w < NW; ++w) cudaStreamSynchronize(ctx->workers[w]->stream);
    };
    auto complete = [&](int w, int k) -> pa_status {
      pa_ctx *wc = ctx->workers[w];
      PendingImage &pi = ws[w].pend[k];
      pi.busy = false;
      if (cudaEventSynchronize(wc->ring_done[k]) != cudaSuccess)
        return fail(ctx, PA_ERR_CUDA, "worker stream: %s", cudaGetErrorString(cudaGetLastError()));
      const pa_status st = finish_complete(wc, ws[w].pend_e[k], pi.pl, pi.outs, pi.rb);
      if (st == PA_ERR_NUMERIC) {
        result = st;
        return PA_OK;
      }
      if (st) ctx->err = wc->err;
      return st;
    };
    for (int g = 0; g < n_groups; ++g) {
      const int w = g % NW, k = ws[w].count % nslots;
      pa_ctx *wc = ctx->workers[w];
      if (ws[w].pend[k].busy)
        if (pa_status st = complete(w, k)) {
          drain();
          return st;
        }
      std::vector<pa_tree> trees;
      std::vector<const float *> ptrs;
      int first = -1;
      for (int i = 0; i < n_images; ++i)
        if (group[i] == g) {
          if (first < 0) first = i;
          trees.push_back(*imgs[i].tree);
          gouts[g].push_back(*imgs[i].out);
          ptrs.push_back(imgs[i].desc);
        }
      const pa_image &f = imgs[first];
      const int n = (int)trees.size();
      ws[w].pend[k].slot = k;
      ws[w].pend_e[k] = f.ep;
      pa_status st = find_obj_core(wc, f.ep, n, trees.data(), f.flip, cls, n_cls, ptrs[0],
                                   ptrs.data(), PA_MEM_DEVICE, f.ny, f.nx, f.dim, f.Tig,
                                   f.tig_shared, f.H, f.W, nullptr, 0,
                                   (int64_t)n * f.ep->num_rotation_steps, gouts[g].data(),
                                   PA_MEM_DEVICE, &ws[w].pend[k]);
      if (st) {
        ctx->err = wc->err;
        drain();
        return st;
      }
      ws[w].pend[k].busy = true;
      ++ws[w].count;
      if (cudaEventRecord(wc->ring_done[k], wc->stream) != cudaSuccess) {
        drain();
        return fail(ctx, PA_ERR_CUDA, "cannot record a worker event");
      }
    }
    pa_status first_err = PA_OK;
    for (int w = 0; w < NW; ++w) {
      pa_ctx *wc = ctx->workers[w];
      if (pa_status st = sync_ctx(wc)) {
        ctx->err = wc->err;
        if (!first_err) first_err = st;
        continue;
      }
      for (int k = 0; k < nslots; ++k)
        if (ws[w].pend[k].busy)
          if (pa_status st = complete(w, k))
            if (!first_err) first_err = st;
      // the worker's launches and kernel times count for the caller's context
      ctx->launches += wc->launches;
      wc->launches = 0;
      for (auto &kv : wc->times) {
        auto &acc = ctx->times[kv.first];
        acc.ms += kv.second.ms;
        acc.n += kv.second.n;
      }
      wc->times.clear();
    }
    return first_err ? first_err : result;
  }
  for (int g = 0; g < n_groups; ++g) {
    std::vector<int> idx;
    for (int i = 0; i < n_images; ++i)
      if (group[i] == g) idx.push_back(i);
    const pa_image &f = imgs[idx[0]];
    std::vector<pa_tree> trees;
    std::vector<pa_ps_outputs> outs;
    std::vector<const float *> ptrs;
    for (int i : idx) {
      trees.push_back(*imgs[i].tree);
      outs.push_back(*imgs[i].out);
      ptrs.push_back(imgs[i].desc);
    }
    const int n = (int)idx.size();
    pa_status st;
    if (mem == PA_MEM_HOST && n > 1)
      st = find_obj_ring(ctx, f.ep, n, trees.data(), f.flip, cls, n_cls, nullptr, ptrs.data(),
                         f.ny, f.nx, f.dim, f.Tig, f.tig_shared, f.H, f.W, nullptr, outs.data());
    else
      st = find_obj_core(ctx, f.ep, n, trees.data(), f.flip, cls, n_cls, ptrs[0],
                         mem == PA_MEM_DEVICE ? ptrs.data() : nullptr, mem, f.ny, f.nx, f.dim,
                         f.Tig, f.tig_shared, f.H, f.W, nullptr, 0,
                         (int64_t)n * f.ep->num_rotation_steps, outs.data(), mem);
    if (st && st != PA_ERR_NUMERIC) return st;
    if (st) result = st;
  }
  return result;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

void pa_queue_opts_default(pa_queue_opts *o) {
  if (!o) return;
  o->images_per_wave = 32;
  o->wait_timeout_ms = 20000.0;
  o->autotune = 1;
  o->hold_start = 0;
}

pa_status pa_find_obj_queue(pa_ctx *ctx, int n_images, const pa_image *imgs,
                            const pa_classifier *const *cls, int n_cls,
                            const pa_queue_opts *opts) try {
  if (!ctx) return PA_ERR_INVALID;
  if (n_images < 0 || (n_images > 0 && (!imgs || !cls || n_cls < 1)))
    return fail(ctx, PA_ERR_INVALID, "invalid image list");
  pa_queue_opts o;
  pa_queue_opts_default(&o);
  if (opts) o = *opts;
  if (o.images_per_wave < 1) o.images_per_wave = 32;
  for (int i = 0; i < n_images; ++i) {
    const pa_image &im = imgs[i];
    if (!im.ep || !exp_ok(im.ep) || !im.tree || !im.desc || !im.Tig || !im.out || im.ny < 1 ||
        im.nx < 1 || im.dim < 1 || im.H < 1 || im.W < 1 || im.H > 32767 || im.W > 32767)
      return fail(ctx, PA_ERR_INVALID, "image %d: invalid sizes, parameters or NULL input", i);
    if (n_scales(im.ep) != 1)
      return fail(ctx, PA_ERR_UNSUPPORTED, "image %d: one scale of descriptors per image", i);
  }
  auto same = [&](const pa_image &a, const pa_image &b) {
    if (std::memcmp(a.ep, b.ep, sizeof(pa_exp_param)) != 0) return false;
    if (a.flip != b.flip || a.ny != b.ny || a.nx != b.nx || a.dim != b.dim || a.H != b.H ||
        a.W != b.W || !a.tig_shared || !b.tig_shared)
      return false;
    return std::memcmp(a.Tig, b.Tig, 9 * sizeof(double)) == 0 && same_topology(a.tree, b.tree);
  };
  DeviceGuard dg(ctx->device);
  pa_status result = PA_OK;
  // Waves alternate between two contexts (the caller's and a worker, each
  // with its own workspace, streams and landing blocks), so that the host
  // plans and queues wave k + 1 while the GPU runs wave k; a context's wave
  // is finished before the context takes the next one.
  const int n_waves = (n_images + o.images_per_wave - 1) / o.images_per_wave;
  pa_ctx *wc[2] = {ctx, nullptr};
  if (n_waves > 1) {
    if (ctx->workers.empty()) {
      pa_ctx *w = nullptr;
      if (pa_ctx_create(ctx->device, &w) != PA_OK)
        return fail(ctx, PA_ERR_CUDA, "cannot create a worker context");
      ctx->workers.push_back(w);
    }
    wc[1] = ctx->workers[0];
    wc[1]->msg_math = ctx->msg_math;
    wc[1]->timing = ctx->timing;
    if (wc[1]->row_tile.empty()) wc[1]->row_tile = ctx->row_tile;
    while (ctx->ring_done.empty()) {
      cudaEvent_t ev;
      PA_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      ctx->ring_done.push_back(ev);
    }
    // the worker starts behind everything queued on the caller's stream
    PA_CK(cudaEventRecord(ctx->ring_done[0], ctx->stream));
    PA_CK(cudaStreamWaitEvent(wc[1]->stream, ctx->ring_done[0], 0));
  }
  std::vector<QGroup> pend[2];
  bool busy[2] = {false, false};
  auto finish = [&](int k) -> pa_status {
    if (!busy[k]) return PA_OK;
    busy[k] = false;
    pa_status st = queue_wave_finish(wc[k], pend[k], o);
    if (st && wc[k] != ctx) ctx->err = wc[k]->err;
    return st;
  };
  auto finish_all = [&]() -> pa_status {
    pa_status st0 = finish(0), st1 = finish(1);
    if (st0 == PA_ERR_NUMERIC) result = st0, st0 = PA_OK;
    if (st1 == PA_ERR_NUMERIC) result = st1, st1 = PA_OK;
    return st0 ? st0 : st1;
  };
  int wave = 0;
  for (int w0 = 0; w0 < n_images; w0 += o.images_per_wave, ++wave) {
    const int w1 = std::min(n_images, w0 + o.images_per_wave);
    const int slot = wave & 1;
    if (pa_status st = finish(slot)) {
      if (st != PA_ERR_NUMERIC) {
        finish_all();
        return st;
      }
      result = st;
    }
    std::vector<QGroup> &groups = pend[slot];
    groups.clear();
    std::vector<int> grp(w1 - w0, -1);
    for (int i = w0; i < w1; ++i) {
      if (grp[i - w0] >= 0) continue;
      grp[i - w0] = (int)groups.size();
      groups.emplace_back();
      for (int j = i + 1; j < w1; ++j)
        if (grp[j - w0] < 0 && same(imgs[i], imgs[j])) grp[j - w0] = grp[i - w0];
    }
    for (int i = w0; i < w1; ++i) {
      QGroup &g = groups[grp[i - w0]];
      if (!g.f) g.f = &imgs[i];
      g.idx.push_back(i);
      g.trees.push_back(*imgs[i].tree);
      g.outs.push_back(*imgs[i].out);
      g.desc.push_back(imgs[i].desc);
      g.marg_out.push_back(imgs[i].out->log_marg);
      g.rp_out.push_back(imgs[i].out->root_post);
    }
    pa_status st = queue_wave(wc[slot], groups, cls, n_cls, o);
    if (st == PA_OK) {
      busy[slot] = true;
      continue;
    }
    if (wc[slot] != ctx) ctx->err = wc[slot]->err;
    // the wave stopped part way (kernels of its unaries may be queued):
    // drain its context, then the other's wave
    cudaStreamSynchronize(wc[slot]->stream);
    for (cudaStream_t ss : wc[slot]->side) cudaStreamSynchronize(ss);
    cudaGetLastError();
    if (pa_status st2 = finish_all()) return st2;
    if (st == PA_ERR_UNSUPPORTED) {
      // a path the queue does not run: this wave as pa_find_obj_multi does it
      st = pa_find_obj_multi(ctx, w1 - w0, imgs + w0, cls, n_cls, PA_MEM_DEVICE);
    }
    if (st == PA_ERR_NUMERIC) {
      result = st;
      continue;
    }
    if (st) return st;
  }
  if (pa_status st = finish_all()) return st;
  return result;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

// ------------------------------------------------------------------------
// Poselet-conditioned extra unaries (objectdetect_findrot.cpp:915-948)
// ------------------------------------------------------------------------
pa_status pa_add_extra_unaries(pa_ctx *ctx, const pa_exp_param *ep, const pa_extra_unary *ex,
                               int n_parts, int root, float *log_unary, int H, int W, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!ep || !exp_ok(ep) || !ex || !log_unary || n_parts < 1 || root < 0 || root >= n_parts ||
      H < 1 || W < 1 || H > 32767 || W > 32767)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes, parameters or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  DeviceGuard dg(ctx->device);
  const int S = n_scales(ep), R = ep->num_rotation_steps;
  const size_t n = (size_t)n_parts * S * R * H * W;
  // getRotScoreGrid's per-rotation table, typed as the reference types it:
  // float rot = rot_from_index / 180 * M_PI, square() in float, exp in
  // double, clipped and logged in float
  std::vector<float> rot_tab((size_t)n_parts * R, 0.f);
  if (ex->rot_params)
    for (int p = 0; p < n_parts; ++p) {
      if (ex->is_detect && !ex->is_detect[p]) continue;
      const float mu = (float)ex->rot_params[2 * p], var = (float)ex->rot_params[2 * p + 1];
      for (int r = 0; r < R; ++r) {
        const float rot = (float)(rot_from_index(ep, r) / 180 * M_PI);
        const float d = rot - mu;
        const float sq = d * d;
        float sc = (float)std::exp(-0.5 * (double)sq / (double)var);
        if ((double)sc < 1e-4) sc = 1e-4f;
        rot_tab[(size_t)p * R + r] = std::log(sc);
      }
    }
  std::vector<float4> pos(n_parts, make_float4(0.f, 0.f, 1.f, 1.f));
  if (ex->pos_params)
    for (int p = 0; p < n_parts; ++p)
      pos[p] = make_float4((float)ex->pos_params[4 * p], (float)ex->pos_params[4 * p + 1],
                           (float)ex->pos_params[4 * p + 2], (float)ex->pos_params[4 * p + 3]);
  std::vector<int> det(n_parts, 1);
  if (ex->is_detect)
    for (int p = 0; p < n_parts; ++p) det[p] = ex->is_detect[p] ? 1 : 0;
  Builder b1;
  b1.param(rot_tab.data(), rot_tab.size());
  b1.param(pos.data(), pos.size());
  b1.param(det.data(), det.size());
  if (mem == PA_MEM_HOST) b1.scratch<float>(n);
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  b.base = ctx->arena;
  ExtraUnary eu{};
  eu.root = root;
  eu.rot_on = ex->rot_params != nullptr;
  eu.pos_on = ex->pos_params != nullptr;
  eu.torso_on = ex->torso_prior != nullptr;
  eu.rot_weight = ex->rot_weight;
  eu.pos_weight = ex->pos_weight;
  eu.torso_weight = ex->torso_weight;
  eu.rot_tab = b.param(rot_tab.data(), rot_tab.size());
  eu.pos = b.param(pos.data(), pos.size());
  eu.is_detect = b.param(det.data(), det.size());
  eu.root_det_x = ex->root_det_x;
  eu.root_det_y = ex->root_det_y;
  if (ex->torso_prior)
    eu.torso = make_float4((float)ex->torso_prior[0], (float)ex->torso_prior[1],
                           (float)ex->torso_prior[2], (float)ex->torso_prior[3]);
  eu.img_cx = (float)(0.5 * W);
  eu.img_cy = (float)(0.5 * H);
  float *d = mem == PA_MEM_HOST ? b.scratch<float>(n) : log_unary;
  if ((st = upload_blob(ctx, b))) return st;
  if (mem == PA_MEM_HOST) PA_CK(cudaMemcpyAsync(d, log_unary, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  PA_LAUNCH("extra_unary", launch_extra_unary(eu, d, n_parts, S, R, H, W, ctx->stream));
  if (mem == PA_MEM_HOST) PA_CK(cudaMemcpyAsync(log_unary, d, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_add_dpm_scores(pa_ctx *ctx, const pa_exp_param *ep, const pa_dpm_terms *dt,
                            int n_parts, int root, float *log_unary, int H, int W, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!ep || !exp_ok(ep) || !dt || !log_unary || n_parts < 1 || root < 0 || root >= n_parts ||
      H < 1 || W < 1 || H > 32767 || W > 32767)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes, parameters or NULL input");
  if (dt->head && (dt->head_part < 0 || dt->head_part >= n_parts))
    return fail(ctx, PA_ERR_INVALID, "head_part out of range");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  DeviceGuard dg(ctx->device);
  const int S = n_scales(ep), R = ep->num_rotation_steps;
  const size_t HW = (size_t)H * W;
  const size_t n = (size_t)n_parts * S * R * HW;
  const size_t n_unary = dt->unary ? (size_t)n_parts * (dt->unary_rot ? R : 1) * HW : 0;
  const size_t n_torso = dt->torso ? HW : 0, n_head = dt->head ? HW : 0;
  std::vector<int> det(n_parts, 1);
  if (dt->is_detect)
    for (int p = 0; p < n_parts; ++p) det[p] = dt->is_detect[p] ? 1 : 0;
  Builder b1;
  b1.param(det.data(), det.size());
  b1.scratch<int>(1);
  if (mem == PA_MEM_HOST) {
    b1.scratch<float>(n);
    b1.scratch<float>(n_torso + n_head + n_unary);
  }
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  b.base = ctx->arena;
  DpmTerms d{};
  d.root = root;
  d.head_part = dt->head_part;
  d.unary_rot = dt->unary_rot ? 1 : 0;
  d.torso_weight = dt->torso_weight;
  d.head_weight = dt->head_weight;
  d.unary_weight = dt->unary_weight;
  d.log_floor = std::log(1e-4);
  d.is_detect = b.param(det.data(), det.size());
  d.err = b.scratch<int>(1);
  float *lu = log_unary, *grids = nullptr;
  if (mem == PA_MEM_HOST) {
    lu = b.scratch<float>(n);
    grids = b.scratch<float>(n_torso + n_head + n_unary);
  }
  if ((st = upload_blob(ctx, b))) return st;
  if (mem == PA_MEM_HOST) {
    PA_CK(cudaMemcpyAsync(lu, log_unary, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    float *g = grids;
    for (auto [src, cnt, dst] : {std::tuple<const float *, size_t, const float **>{dt->torso, n_torso, &d.torso},
                                 {dt->head, n_head, &d.head}, {dt->unary, n_unary, &d.unary}}) {
      if (!src) continue;
      PA_CK(cudaMemcpyAsync(g, src, cnt * 4, cudaMemcpyHostToDevice, ctx->stream));
      *dst = g;
      g += cnt;
    }
  } else {
    d.torso = dt->torso;
    d.head = dt->head;
    d.unary = dt->unary;
  }
  PA_CK(cudaMemsetAsync(d.err, 0, sizeof(int), ctx->stream));
  PA_LAUNCH("dpm_score", launch_dpm_score(d, lu, n_parts, S, R, H, W, ctx->stream));
  int flag = 0;
  PA_CK(cudaMemcpyAsync(&flag, d.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (mem == PA_MEM_HOST) PA_CK(cudaMemcpyAsync(log_unary, lu, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (pa_status ss = sync_ctx(ctx)) return ss;
  // computeLogGrid asserts data >= 0 (multi_array_op.hpp:154-167)
  if (flag) return fail(ctx, PA_ERR_INVALID, "negative or NaN torso DPM score");
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_nms_rects(pa_ctx *ctx, int n, const double *rects, const double *score,
                       double ellipse_size, int *suppressed, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (n < 0 || n > PA_NMS_MAX_HYPS || (n > 0 && (!rects || !score || !suppressed)))
    return fail(ctx, PA_ERR_INVALID, "invalid rectangle count or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  if (n == 0) return PA_OK;
  DeviceGuard dg(ctx->device);
  Builder b1;
  b1.scratch<int>(1);
  if (mem == PA_MEM_HOST) {
    b1.scratch<double>((size_t)9 * n);
    b1.scratch<int>(n);
  }
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  b.base = ctx->arena;
  int *err = b.scratch<int>(1);
  cudaStream_t s = ctx->stream;
  const double *dr = rects, *dsc = score;
  int *dout = suppressed;
  if (mem == PA_MEM_HOST) {
    double *h = b.scratch<double>((size_t)9 * n);
    dout = b.scratch<int>(n);
    PA_CK(cudaMemcpyAsync(h, rects, (size_t)8 * n * sizeof(double), cudaMemcpyHostToDevice, s));
    PA_CK(cudaMemcpyAsync(h + (size_t)8 * n, score, (size_t)n * sizeof(double),
                          cudaMemcpyHostToDevice, s));
    dr = h;
    dsc = h + (size_t)8 * n;
  }
  // square(ellipse_size) * dist_threshold, dist_threshold = 1 (nms.cpp:135-158)
  const double thr = (ellipse_size * ellipse_size) * 1.0;
  PA_CK(cudaMemsetAsync(err, 0, sizeof(int), s));
  PA_LAUNCH("nms", launch_nms_rects(dr, dsc, n, thr, dout, err, s));
  int flag = 0;
  PA_CK(cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (mem == PA_MEM_HOST)
    PA_CK(cudaMemcpyAsync(suppressed, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  if (pa_status ss = sync_ctx(ctx)) return ss;
  if (flag) return fail(ctx, PA_ERR_INVALID, "unsorted hypothesis vector");
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

void pa_rect_from_hyp(float x, float y, float scale, double reference_height,
                      double reference_width, double *rect) {
  if (!rect) return;
  const int h = (int)((double)scale * reference_height);
  const int w = (int)((double)scale * reference_width);
  const double c = 1.0, sn = 0.0;  // upright rectangles only, as the reference
  const double v1x = c * w / 2, v1y = sn * w / 2;
  const double v2x = -sn * h / 2, v2y = c * h / 2;
  const double px = (double)x, py = (double)y;
  const double pts[4][2] = {{(px - v1x) - v2x, (py - v1y) - v2y},
                            {(px + v1x) - v2x, (py + v1y) - v2y},
                            {(px + v1x) + v2x, (py + v1y) + v2y},
                            {(px - v1x) + v2x, (py - v1y) + v2y}};
  for (int k = 0; k < 4; ++k) {
    rect[2 * k] = pts[k][0];
    rect[2 * k + 1] = pts[k][1];
  }
}

pa_status pa_nms_recursive(pa_ctx *ctx, int n, const float *x, const float *y, const float *scale,
                           const float *score, double train_object_width,
                           double train_object_height, int *suppressed, int mem) try {
  if (!ctx) return PA_ERR_INVALID;
  if (n < 0 || n > PA_NMS_MAX_HYPS || (n > 0 && (!x || !y || !scale || !score || !suppressed)) ||
      !(train_object_width > 0) || !(train_object_height > 0))
    return fail(ctx, PA_ERR_INVALID, "invalid hypothesis count, sizes or NULL input");
  if (mem != PA_MEM_DEVICE && mem != PA_MEM_HOST) return fail(ctx, PA_ERR_INVALID, "bad mem");
  if (n == 0) return PA_OK;
  DeviceGuard dg(ctx->device);
  Builder b1;
  b1.scratch<int>(1);
  if (mem == PA_MEM_HOST) {
    b1.scratch<float>((size_t)4 * n);
    b1.scratch<int>(n);
  }
  pa_status st = ensure_arena(ctx, b1.total());
  if (st) return st;
  Builder b;
  b.dry = false;
  b.blob_size = b1.blob.size();
  b.base = ctx->arena;
  int *err = b.scratch<int>(1);
  cudaStream_t s = ctx->stream;
  const float *dx = x, *dy = y, *ds = scale, *dsc = score;
  int *dout = suppressed;
  if (mem == PA_MEM_HOST) {
    float *h = b.scratch<float>((size_t)4 * n);
    dout = b.scratch<int>(n);
    const float *src[4] = {x, y, scale, score};
    for (int k = 0; k < 4; ++k)
      PA_CK(cudaMemcpyAsync(h + (size_t)k * n, src[k], (size_t)n * 4, cudaMemcpyHostToDevice, s));
    dx = h;
    dy = h + n;
    ds = h + 2 * (size_t)n;
    dsc = h + 3 * (size_t)n;
  }
  PA_CK(cudaMemsetAsync(err, 0, sizeof(int), s));
  PA_LAUNCH("nms", launch_nms(dx, dy, ds, dsc, n, train_object_width, train_object_height, dout, err, s));
  int flag = 0;
  PA_CK(cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (mem == PA_MEM_HOST)
    PA_CK(cudaMemcpyAsync(suppressed, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  if (pa_status ss = sync_ctx(ctx)) return ss;
  if (flag) return fail(ctx, PA_ERR_INVALID, "unsorted hypothesis vector");
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

// ------------------------------------------------------------------------
// Learned unary
// ------------------------------------------------------------------------
pa_status pa_unary_net_create(pa_ctx *ctx, int dim, int n_parts, uint64_t seed,
                              pa_unary_net **out) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!out || dim < 64 || dim % 64 || dim > 4096 || n_parts < 1 || n_parts > 64)
    return fail(ctx, PA_ERR_INVALID, "net: dim must be a multiple of 64 (<= 4096), 1 <= n_parts <= 64");
  *out = nullptr;
  DeviceGuard dg(ctx->device);
  pa_unary_net *net = new pa_unary_net;
  net->device = ctx->device;
  net->dim = dim;
  net->P = n_parts;
  net_layout(net);
  const size_t np = (size_t)net->n_params;
  const size_t bytes = np * 16 + ((size_t)64 * dim + 8 * 64 * 576) * 2 + 256;
  char *base = nullptr;
  if (cudaMalloc(&base, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete net;
    return fail(ctx, PA_ERR_NOMEM, "cannot allocate %zu bytes for the unary net", bytes);
  }
  net->params = reinterpret_cast<float *>(base);
  net->grads = net->params + np;
  net->adam_m = net->grads + np;
  net->adam_v = net->adam_m + np;
  __nv_bfloat16 *w = reinterpret_cast<__nv_bfloat16 *>(net->adam_v + np);
  net->wf0 = w;
  w += (size_t)64 * dim;
  for (int l = 0; l < 4; ++l, w += 64 * 576) net->wf[l] = w;
  for (int l = 0; l < 4; ++l, w += 64 * 576) net->wd[l] = w;
  net->err = reinterpret_cast<int *>(w);
  // He-normal weights from splitmix64 + Box-Muller (the output layer at a
  // tenth of that, so that its first predictions are close to its bias),
  // zero biases
  std::vector<float> h(np, 0.f);
  uint64_t st = seed ^ 0x6a09e667f3bcc909ull;
  auto next = [&]() {
    uint64_t z = (st += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  };
  auto unit = [&]() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  for (int l = 0; l < 5; ++l) {
    const double sd = std::sqrt(2.0 / (l == 0 ? dim : 576)) * (l == 4 ? 0.1 : 1.0);
    for (int64_t i = net->off_w[l]; i < net->off_b[l]; i += 2) {
      const double r = std::sqrt(-2.0 * std::log(unit())), t = 2.0 * M_PI * unit();
      h[i] = (float)(sd * r * std::cos(t));
      if (i + 1 < net->off_b[l]) h[i + 1] = (float)(sd * r * std::sin(t));
    }
  }
  *out = net;
  pa_status s = pa_unary_net_set_params(ctx, net, h.data());
  if (s) {
    pa_unary_net_destroy(ctx, net);
    *out = nullptr;
  }
  return s;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_net_destroy(pa_ctx *ctx, pa_unary_net *net) try {
  if (!net) return PA_OK;
  DeviceGuard dg(net->device);
  if (ctx && ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (net->scratch) cudaFree(net->scratch);
  if (net->params) cudaFree(net->params);
  delete net;
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_net_get_params(pa_ctx *ctx, const pa_unary_net *net, float *params,
                                  int64_t *n_params) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!net) return fail(ctx, PA_ERR_INVALID, "NULL net");
  if (n_params) *n_params = net->n_params;
  if (!params) return PA_OK;
  DeviceGuard dg(ctx->device);
  PA_CK(cudaMemcpyAsync(params, net->params, (size_t)net->n_params * 4, cudaMemcpyDeviceToHost,
                        ctx->stream));
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_net_set_params(pa_ctx *ctx, pa_unary_net *net, const float *params) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!net || !params) return fail(ctx, PA_ERR_INVALID, "NULL net or parameters");
  DeviceGuard dg(ctx->device);
  const size_t np = (size_t)net->n_params;
  PA_CK(cudaMemcpyAsync(net->params, params, np * 4, cudaMemcpyHostToDevice, ctx->stream));
  PA_CK(cudaMemsetAsync(net->grads, 0, np * 12, ctx->stream));  // grads, Adam m and v
  PA_CK(cudaMemsetAsync(net->err, 0, sizeof(int), ctx->stream));
  net->step = 0;
  if (pa_status st = net_pack(ctx, net)) return st;
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_net_forward(pa_ctx *ctx, pa_unary_net *net, const void *fields, int fields_bf16,
                               int n_fields, int ny, int nx, float *out, int64_t out_field_stride,
                               int64_t out_part_stride, int exp_out) try {
  if (!ctx) return PA_ERR_INVALID;
  if (pa_status st = net_check_fields(ctx, net, fields, n_fields, ny, nx)) return st;
  if (!out) return fail(ctx, PA_ERR_INVALID, "NULL output");
  DeviceGuard dg(ctx->device);
  NetScratch sc;
  if (pa_status st = net_scratch(ctx, net, n_fields, ny, nx, !fields_bf16, false, sc)) return st;
  PA_CK(cudaMemsetAsync(net->err, 0, sizeof(int), ctx->stream));
  if (pa_status st = net_forward(ctx, net, fields, fields_bf16 ? 1 : 0, n_fields, ny, nx, out,
                                 out_field_stride, out_part_stride, exp_out ? 1 : 0, sc))
    return st;
  return net_err_check(ctx, net);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_net_backward(pa_ctx *ctx, pa_unary_net *net, const void *fields,
                                int fields_bf16, const float *scores, int n_fields, int ny,
                                int nx, double *loss, float *grads) try {
  if (!ctx) return PA_ERR_INVALID;
  if (pa_status st = net_check_fields(ctx, net, fields, n_fields, ny, nx)) return st;
  if (!scores) return fail(ctx, PA_ERR_INVALID, "NULL scores");
  DeviceGuard dg(ctx->device);
  NetScratch sc;
  if (pa_status st = net_scratch(ctx, net, n_fields, ny, nx, !fields_bf16, true, sc)) return st;
  PA_CK(cudaMemsetAsync(net->err, 0, sizeof(int), ctx->stream));
  if (pa_status st = net_backward(ctx, net, fields, fields_bf16 ? 1 : 0, scores, n_fields, ny, nx, sc))
    return st;
  double l = 0.0;
  PA_CK(cudaMemcpyAsync(&l, sc.loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (grads)
    PA_CK(cudaMemcpyAsync(grads, net->grads, (size_t)net->n_params * 4, cudaMemcpyDeviceToHost,
                          ctx->stream));
  if (pa_status st = net_err_check(ctx, net)) return st;
  if (loss) *loss = l * (1.0 / ((double)n_fields * ny * nx * net->P));
  return PA_OK;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_unary_net_adam(pa_ctx *ctx, pa_unary_net *net, const pa_adam_param *opt) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!net || !opt || !(opt->lr >= 0.f) || !(opt->beta1 >= 0.f && opt->beta1 < 1.f) ||
      !(opt->beta2 >= 0.f && opt->beta2 < 1.f) || !(opt->eps > 0.f))
    return fail(ctx, PA_ERR_INVALID, "invalid Adam parameters");
  DeviceGuard dg(ctx->device);
  net->step += 1;
  AdamArgs a{};
  a.lr = opt->lr;
  a.b1 = opt->beta1;
  a.b2 = opt->beta2;
  a.eps = opt->eps;
  a.bc1 = (float)(1.0 - std::pow((double)opt->beta1, (double)net->step));
  a.bc2 = (float)(1.0 - std::pow((double)opt->beta2, (double)net->step));
  PA_LAUNCH("net_adam", launch_adam(net->params, net->grads, net->adam_m, net->adam_v,
                                    net->n_params, a, ctx->stream));
  if (pa_status st = net_pack(ctx, net)) return st;
  return sync_ctx(ctx);
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

pa_status pa_find_obj_batch_learned(pa_ctx *ctx, const pa_exp_param *ep, int n_images,
                                    const pa_tree *trees, int flip, pa_unary_net *net,
                                    const int *part_on_net, const pa_classifier *const *cls,
                                    int n_cls, const void *fields, const float *desc, int ny,
                                    int nx, int dim, const double *Tig, int tig_shared, int H,
                                    int W, const pa_ps_outputs *out) try {
  if (!ctx) return PA_ERR_INVALID;
  if (!ep || !exp_ok(ep)) return fail(ctx, PA_ERR_INVALID, "invalid experiment parameters");
  if (n_scales(ep) != 1)
    return fail(ctx, PA_ERR_UNSUPPORTED,
                "the descriptors are one scale; pa_find_obj_scales takes several");
  if (!net || n_images < 1 || !trees || !Tig || !out || ny < 1 || nx < 1 || dim != net->dim ||
      H < 1 || W < 1 || H > 32767 || W > 32767 || trees[0].n_parts != net->P)
    return fail(ctx, PA_ERR_INVALID, "invalid sizes, NULL input, or a net of another shape");
  LearnedUnary lu;
  lu.net = net;
  lu.fields = fields;
  lu.on_net.assign(net->P, 1);
  if (part_on_net)
    for (int p = 0; p < net->P; ++p) lu.on_net[p] = part_on_net[p] ? 1 : 0;
  for (int p = 0; p < net->P; ++p) (lu.on_net[p] ? lu.any_net : lu.any_ada) = true;
  if (lu.any_net && (!fields || ((uintptr_t)fields & 15)))
    return fail(ctx, PA_ERR_INVALID, "the net's parts need BF16 fields (16-byte aligned)");
  if (lu.any_ada && (!desc || !cls || n_cls < net->P))
    return fail(ctx, PA_ERR_INVALID, "the AdaBoost parts need FP32 descriptors and classifiers");
  DeviceGuard dg(ctx->device);
  pa_status st = find_obj_core(ctx, ep, n_images, trees, flip, cls, net->P,
                               desc, nullptr, PA_MEM_DEVICE, ny, nx, dim, Tig, tig_shared, H, W,
                               nullptr, 0, (int64_t)n_images * ep->num_rotation_steps, out,
                               PA_MEM_DEVICE, nullptr, &lu);
  if (st && st != PA_ERR_NUMERIC) return st;
  if (lu.any_net)
    if (pa_status s2 = net_err_check(ctx, net)) return s2;
  return st;
} catch (const std::bad_alloc &) {
  return fail(ctx, PA_ERR_NOMEM, "host memory exhausted");
} catch (const std::exception &exc) {
  return fail(ctx, PA_ERR_INVALID, "%s", exc.what());
}

}  // extern "C"
