// objectdetect_gpu.cpp -- the reference-shaped host functions of
// partapp_gpu.hpp, each a thin adapter onto include/partapp_gb300.h.
#include "partapp_gpu.hpp"

#include <algorithm>
#include <cctype>
#include <fstream>
#include <cstdio>
#include <cstring>

#include "mat_io.hpp"

namespace partapp_gpu {

namespace {

// The C-ABI view of a tree: arrays kept alive by the holder.
struct TreeHolder {
  std::vector<int> is_upright, child, parent;
  std::vector<double> oc, op, C, rot_mean, rot_sigma;
  pa_tree t{};

  TreeHolder(const PartConfig &pc, int root, const std::vector<Joint> &joints) {
    is_upright = pc.is_upright;
    for (const Joint &j : joints) {
      child.push_back(j.child_idx);
      parent.push_back(j.parent_idx);
      oc.insert(oc.end(), j.offset_c, j.offset_c + 2);
      op.insert(op.end(), j.offset_p, j.offset_p + 2);
      C.insert(C.end(), j.C, j.C + 4);
      rot_mean.push_back(j.rot_mean);
      rot_sigma.push_back(j.rot_sigma);
    }
    t.n_parts = pc.part_size();
    t.root = root;
    t.is_upright = is_upright.data();
    t.n_joints = (int)joints.size();
    t.child = child.data();
    t.parent = parent.data();
    t.offset_c = oc.data();
    t.offset_p = op.data();
    t.C = C.data();
    t.rot_mean = rot_mean.data();
    t.rot_sigma = rot_sigma.data();
  }
};

PartHyp to_hyp(const pa_part_hyp &h) {
  PartHyp p;
  p.m_scaleidx = (int)h.scaleidx;
  p.m_scale = h.scale;
  p.m_rotidx = (int)h.rotidx;
  p.m_rot = h.rot;
  p.m_x = (int)h.x;
  p.m_y = (int)h.y;
  p.m_score = h.score;
  return p;
}

void require(bool ok, const std::string &what) {
  if (!ok) throw Error(PA_ERR_INVALID, what);
}

// Output buffers of one image.
struct ImageOut {
  std::vector<pa_part_hyp> best, part_hyps;
  std::vector<int> n_part_hyps;
  std::vector<float> root_hyps;
  int n_root_hyps = 0;
  std::vector<double> log_z;
  pa_ps_outputs o{};

  ImageOut(int P, int K, int S = 1)
      : best(P), part_hyps((size_t)P * K), n_part_hyps(P), root_hyps(1000 * 4), log_z((size_t)S * P) {
    o.best = best.data();
    o.part_hyps = part_hyps.data();
    o.n_part_hyps = n_part_hyps.data();
    o.root_hyps = root_hyps.data();
    o.n_root_hyps = &n_root_hyps;
    o.log_z = log_z.data();
  }

  FindObjResult result(int P, int K) const {
    FindObjResult r;
    for (int p = 0; p < P; ++p) r.best_conf.push_back(to_hyp(best[p]));
    r.part_hyps.resize(P);
    for (int p = 0; p < P; ++p)
      for (int k = 0; k < n_part_hyps[p]; ++k) r.part_hyps[p].push_back(to_hyp(part_hyps[(size_t)p * K + k]));
    for (int k = 0; k < n_root_hyps; ++k)
      r.root_hyps.push_back(std::vector<float>(root_hyps.begin() + 4 * k, root_hyps.begin() + 4 * k + 4));
    r.log_z = log_z;
    return r;
  }
};

}  // namespace

pa_exp_param ExpParam::c() const {
  pa_exp_param e;
  pa_exp_param_default(&e);
  e.num_rotation_steps = num_rotation_steps;
  e.min_part_rotation = min_part_rotation;
  e.max_part_rotation = max_part_rotation;
  e.min_object_scale = min_object_scale;
  e.max_object_scale = max_object_scale;
  e.strip_border_detections = strip_border_detections;
  e.roi_save_num_samples = roi_save_num_samples;
  e.use_pairwise = use_pairwise ? 1 : 0;
  e.interpolate = interpolate ? 1 : 0;
  e.num_scale_steps = num_scale_steps;
  return e;
}

std::vector<float> PartHyp::toVect() const {
  return {(float)m_scaleidx, (float)m_scale, (float)m_rotidx, (float)m_rot,
          (float)m_x,        (float)m_y,     m_score};
}

Context::Context(int device) {
  const pa_status s = pa_ctx_create(device, &ctx_);
  if (s != PA_OK) throw Error(s, std::string("pa_ctx_create: ") + pa_status_string(s));
}

Context::~Context() {
  if (ctx_) pa_ctx_destroy(ctx_);
}

void Context::check(pa_status s) const {
  if (s != PA_OK) throw Error(s, std::string(pa_status_string(s)) + ": " + pa_last_error(ctx_));
}

AdaBoostClassifier::AdaBoostClassifier(Context &ctx, const std::string &text) : ctx_(ctx) {
  ctx.check(pa_classifier_parse(ctx.get(), text.data(), text.size(), &cls_));
}

AdaBoostClassifier::AdaBoostClassifier(Context &ctx, int dim, const std::vector<pa_stump> &stumps)
    : ctx_(ctx) {
  ctx.check(pa_classifier_create(ctx.get(), dim, stumps.data(), (int)stumps.size(), &cls_));
}

AdaBoostClassifier::~AdaBoostClassifier() {
  if (cls_) pa_classifier_destroy(ctx_.get(), cls_);
}

int AdaBoostClassifier::dim() const {
  int d = 0;
  pa_classifier_info(cls_, &d, nullptr, nullptr);
  return d;
}

int AdaBoostClassifier::size() const {
  int n = 0;
  pa_classifier_info(cls_, nullptr, &n, nullptr);
  return n;
}

float AdaBoostClassifier::sum_alpha() const {
  float s = 0;
  pa_classifier_info(cls_, nullptr, nullptr, &s);
  return s;
}

void computeRotJointMarginal(Context &ctx, const ExpParam &exp_param, FloatGrid3 &log_prob_child,
                             FloatGrid3 &log_prob_parent, const double offset_c_10[2],
                             const double offset_p_01[2], const double C[4], double rot_mean,
                             double rot_sigma, double scale, bool bIsSparse) {
  const size_t *s = log_prob_child.shape();
  if (log_prob_parent.num_elements() != log_prob_child.num_elements())
    log_prob_parent = FloatGrid3(s[0], s[1], s[2]);
  const pa_exp_param e = exp_param.c();
  ctx.check(pa_rot_joint_marginal(ctx.get(), &e, log_prob_child.data(), log_prob_parent.data(),
                                  (int)s[0], (int)s[1], (int)s[2], offset_c_10, offset_p_01, C,
                                  rot_mean, rot_sigma, scale, bIsSparse ? 1 : 0, PA_MEM_HOST));
}

void computeRootPosteriorRot(Context &ctx, const PartApp &part_app,
                             std::vector<std::vector<FloatGrid3>> &log_part_detections,
                             FloatGrid3 &root_part_posterior, int rootpart_idx,
                             std::vector<Joint> joints, bool flip, bool bIsSparse, int imgidx,
                             std::vector<std::vector<PartHyp>> &best_part_hyp,
                             bool bSaveMarginals, std::vector<FloatGrid3> *log_marginals,
                             std::vector<double> *log_z) {
  (void)flip;  // the joints are already mirrored by loadJoints; flip only names output files
  (void)imgidx;
  (void)bSaveMarginals;
  const int P = (int)log_part_detections.size();
  require(P == part_app.m_part_conf.part_size(), "one detection stack per part");
  require(P > 0 && !log_part_detections[0].empty(), "empty detections");
  const pa_exp_param e = part_app.m_exp_param.c();
  const int S = (int)log_part_detections[0].size();
  require(S == std::max(1, e.num_scale_steps), "one map per scale (num_scale_steps)");
  const size_t *s = log_part_detections[0][0].shape();
  const int R = (int)s[0], H = (int)s[1], W = (int)s[2];
  const size_t N = (size_t)R * H * W;
  std::vector<float> unary((size_t)P * S * N);  // [part][scale][R][H][W]
  for (int p = 0; p < P; ++p)
    for (int sc = 0; sc < S; ++sc) {
      require((int)log_part_detections[p].size() == S &&
                  log_part_detections[p][sc].num_elements() == N,
              "all parts need [R][H][W] maps of one size at every scale");
      std::memcpy(unary.data() + ((size_t)p * S + sc) * N, log_part_detections[p][sc].data(),
                  N * sizeof(float));
    }
  const TreeHolder th(part_app.m_part_conf, rootpart_idx, joints);
  const int K = e.roi_save_num_samples;
  ImageOut out(P, K > 0 ? K : 1, S);
  root_part_posterior = FloatGrid3(S, H, W);  // [nScales][H][W], :718
  out.o.root_post = root_part_posterior.data();
  std::vector<float> marg;
  if (log_marginals) {
    marg.resize((size_t)P * S * N);
    out.o.log_marg = marg.data();
  }
  ctx.check(pa_ps_infer(ctx.get(), &e, &th.t, 0, bIsSparse ? 1 : 0, unary.data(), H, W, &out.o,
                        PA_MEM_HOST));
  const FindObjResult r = out.result(P, K > 0 ? K : 1);
  // best_part_hyp[p] = the argmax, then the local maxima (objectdetect_findrot.cpp:276-283)
  best_part_hyp.assign(P, {});
  for (int p = 0; p < P; ++p) {
    best_part_hyp[p].push_back(r.best_conf[p]);
    best_part_hyp[p].insert(best_part_hyp[p].end(), r.part_hyps[p].begin(), r.part_hyps[p].end());
  }
  if (log_marginals) {
    log_marginals->clear();
    for (size_t k = 0; k < (size_t)P * S; ++k) {
      FloatGrid3 g(R, H, W);
      std::memcpy(g.data(), marg.data() + k * N, N * sizeof(float));
      log_marginals->push_back(std::move(g));
    }
  }
  if (log_z) *log_z = r.log_z;
}

void computeScoreGrids(Context &ctx, const std::vector<const AdaBoostClassifier *> &abc,
                       const float *desc, int n_fields, int ny, int nx, int dim,
                       bool bNormalizeBoost, std::vector<FloatGrid3> &scores) {
  std::vector<const pa_classifier *> cls;
  for (const AdaBoostClassifier *a : abc) cls.push_back(a->get());
  const size_t per = (size_t)n_fields * ny * nx;
  std::vector<float> buf(cls.size() * per);
  ctx.check(pa_score_grids(ctx.get(), cls.data(), (int)cls.size(), desc, n_fields, ny, nx, dim,
                           bNormalizeBoost ? 1 : 0, buf.data(), PA_MEM_HOST));
  scores.clear();
  for (size_t c = 0; c < cls.size(); ++c) {
    FloatGrid3 g(n_fields, ny, nx);
    std::memcpy(g.data(), buf.data() + c * per, per * sizeof(float));
    scores.push_back(std::move(g));
  }
}

FindObjResult findObjectImageRotJoints(Context &ctx, const PartApp &part_app, bool flip,
                                       const float *desc, int ny, int nx, int dim,
                                       const double Tig[9], int H, int W, bool want_marginals) {
  return findObjectDataset(ctx, part_app, flip, {part_app.m_joints}, desc, 1, ny, nx, dim, Tig, H,
                           W, want_marginals)[0];
}

namespace {

std::vector<float> partdetect_raw(Context &ctx, const PartApp &part_app, const float *image,
                                  int img_h, int img_w, bool flip) {
  const pa_exp_param e = part_app.m_exp_param.c();
  const int n = (int)part_app.m_abc.size();
  require(n > 0 && (int)part_app.m_window_param.size() == n, "one window per classifier");
  std::vector<const pa_classifier *> cls;
  for (const AdaBoostClassifier *a : part_app.m_abc) cls.push_back(a->get());
  std::vector<pa_part_window> wins(n);
  for (int c = 0; c < n; ++c) {
    const PartWindow &w = part_app.m_window_param[c];
    wins[c] = {w.window_size_x, w.window_size_y, w.pos_offset_x, w.pos_offset_y};
  }
  const pa_abc_param abc = {part_app.m_abc_param.desc_step, part_app.m_abc_param.desc_size,
                            part_app.m_abc_param.window_desc_step_ratio};
  const int S = std::max(1, e.num_scale_steps), R = e.num_rotation_steps;
  const std::vector<float> *mask = part_app.m_detection_mask;
  require(!mask || mask->size() == (size_t)S * img_h * img_w, "detection masks: [S][H][W]");
  std::vector<float> lu((size_t)n * S * R * img_h * img_w);
  ctx.check(pa_partdetect_masked(ctx.get(), &e, image, img_h, img_w, flip ? 1 : 0, cls.data(),
                                 n, wins.data(), &abc, mask ? mask->data() : nullptr, lu.data(),
                                 PA_MEM_HOST));
  return lu;
}

// Adds part_app.m_extra's terms to the host log unaries [P][S][R][H][W].
void applyExtraUnaries(Context &ctx, const PartApp &part_app, std::vector<float> &lu, int H,
                       int W) {
  const ExtraUnaryParams *x = part_app.m_extra;
  if (!x) return;
  const pa_exp_param e = part_app.m_exp_param.c();
  const int P = part_app.m_part_conf.part_size();
  const int R = e.num_rotation_steps;
  const size_t HW = (size_t)H * W;
  if (!x->dpm_torso.empty() || !x->dpm_head.empty() || !x->dpm_unary.empty()) {
    require(x->dpm_torso.empty() || x->dpm_torso.size() == HW, "DPM torso grid: [H][W]");
    require(x->dpm_head.empty() || x->dpm_head.size() == HW, "DPM head grid: [H][W]");
    require(x->dpm_unary.empty() ||
                x->dpm_unary.size() == (size_t)P * (x->dpm_unary_rot ? R : 1) * HW,
            "DPM unary grids: [P][R or 1][H][W]");
    pa_dpm_terms dt{};
    dt.torso_weight = x->dpm_torso_weight;
    dt.torso = x->dpm_torso.empty() ? nullptr : x->dpm_torso.data();
    dt.head_weight = x->dpm_head_weight;
    dt.head_part = x->dpm_head_part;
    dt.head = x->dpm_head.empty() ? nullptr : x->dpm_head.data();
    dt.unary_weight = x->dpm_unary_weight;
    dt.unary_rot = x->dpm_unary_rot;
    dt.unary = x->dpm_unary.empty() ? nullptr : x->dpm_unary.data();
    dt.is_detect = x->is_detect.empty() ? nullptr : x->is_detect.data();
    ctx.check(pa_add_dpm_scores(ctx.get(), &e, &dt, P, part_app.m_part_conf.rootpart_idx,
                                lu.data(), H, W, PA_MEM_HOST));
  }
  if (x->rot.empty() && x->pos.empty() && x->torso.empty()) return;
  require(x->rot.empty() || (int)x->rot.size() == 2 * P, "rotation parameters: 2 per part");
  require(x->pos.empty() || (int)x->pos.size() == 4 * P, "position parameters: 4 per part");
  require(x->torso.empty() || x->torso.size() == 4, "torso prior: 4 parameters");
  require(x->is_detect.empty() || (int)x->is_detect.size() == P, "is_detect: one flag per part");
  pa_extra_unary ex{};
  ex.rot_weight = x->rot_weight;
  ex.rot_params = x->rot.empty() ? nullptr : x->rot.data();
  ex.pos_weight = x->pos_weight;
  ex.pos_params = x->pos.empty() ? nullptr : x->pos.data();
  ex.root_det_x = x->root_det_x;
  ex.root_det_y = x->root_det_y;
  ex.torso_weight = x->torso_weight;
  ex.torso_prior = x->torso.empty() ? nullptr : x->torso.data();
  ex.is_detect = x->is_detect.empty() ? nullptr : x->is_detect.data();
  ctx.check(pa_add_extra_unaries(ctx.get(), &e, &ex, P, part_app.m_part_conf.rootpart_idx,
                                 lu.data(), H, W, PA_MEM_HOST));
}

}  // namespace

void partdetect(Context &ctx, const PartApp &part_app, const float *image, int img_h,
                int img_w, bool flip, std::vector<std::vector<FloatGrid3>> &log_part_detections) {
  const pa_exp_param e = part_app.m_exp_param.c();
  const int n = (int)part_app.m_abc.size();
  const int S = std::max(1, e.num_scale_steps), R = e.num_rotation_steps;
  const std::vector<float> lu = partdetect_raw(ctx, part_app, image, img_h, img_w, flip);
  const size_t N = (size_t)R * img_h * img_w;
  log_part_detections.assign(n, std::vector<FloatGrid3>());
  for (int c = 0; c < n; ++c)
    for (int sc = 0; sc < S; ++sc) {
      FloatGrid3 g(R, img_h, img_w);
      std::memcpy(g.data(), lu.data() + ((size_t)c * S + sc) * N, N * sizeof(float));
      log_part_detections[c].push_back(std::move(g));
    }
}

FindObjResult findObjectImageFromImage(Context &ctx, const PartApp &part_app, bool flip,
                                       const std::vector<Joint> &joints, const float *image,
                                       int img_h, int img_w, bool want_marginals) {
  const pa_exp_param e = part_app.m_exp_param.c();
  const int P = part_app.m_part_conf.part_size();
  require((int)part_app.m_abc.size() >= P, "a detector for every part");
  const int S = std::max(1, e.num_scale_steps), R = e.num_rotation_steps;
  // partdetect(part_app, imgidx, imgidx, false /* flip */, ...), objectdetect_aux.cpp:383
  std::vector<float> lu = partdetect_raw(ctx, part_app, image, img_h, img_w, false);
  // the first P classifiers' unaries are the parts' [P][S][R][H][W] block
  applyExtraUnaries(ctx, part_app, lu, img_h, img_w);
  const TreeHolder th(part_app.m_part_conf, part_app.m_part_conf.rootpart_idx, joints);
  const int K = e.roi_save_num_samples > 0 ? e.roi_save_num_samples : 1;
  ImageOut out(P, K, S);
  const size_t N = (size_t)R * img_h * img_w;
  std::vector<float> marg;
  if (want_marginals) {
    marg.resize((size_t)P * S * N);
    out.o.log_marg = marg.data();
  }
  // the first P classifiers' unaries are the leading [P][S][R][H][W] block
  ctx.check(pa_ps_infer(ctx.get(), &e, &th.t, flip ? 1 : 0, 1, lu.data(), img_h, img_w, &out.o,
                        PA_MEM_HOST));
  FindObjResult r = out.result(P, K);
  if (want_marginals)
    for (size_t k = 0; k < (size_t)P * S; ++k) {
      FloatGrid3 g(R, img_h, img_w);
      std::memcpy(g.data(), marg.data() + k * N, N * sizeof(float));
      r.log_marginals.push_back(std::move(g));
    }
  return r;
}

ExtraUnaryParams loadExtraUnaryParams(int imgidx, int n_parts, int root, const std::string &pred_dir,
                                      float rot_weight, float pos_weight,
                                      const std::string &torso_det_dir, int rootidx_det,
                                      const std::string &torso_prior_file, float torso_weight) {
  ExtraUnaryParams x;
  if (!pred_dir.empty() && rot_weight != 0.f) {
    const auto v = mat_read(pred_dir + "/testlist_params_rot_imgidx_" + std::to_string(imgidx) + ".mat");
    const MatArray &a = mat_find(v, "rot_test");
    require(a.dims.size() == 2 && (int)a.dims[0] >= n_parts && a.dims[1] >= 2, "rot_test: [P][2+]");
    x.rot_weight = rot_weight;
    for (int p = 0; p < n_parts; ++p) {
      const double sd = mat_at(a, {(size_t)p, 1});
      x.rot.push_back(mat_at(a, {(size_t)p, 0}));
      x.rot.push_back(sd * sd);  // square()
    }
  }
  if (!pred_dir.empty() && pos_weight != 0.f) {
    const auto v = mat_read(pred_dir + "/testlist_params_pos_imgidx_" + std::to_string(imgidx) + ".mat");
    const MatArray &a = mat_find(v, "pos_test");
    require(a.dims.size() == 2 && (int)a.dims[0] >= n_parts && a.dims[1] >= 4, "pos_test: [P][4+]");
    x.pos_weight = pos_weight;
    for (int p = 0; p < n_parts; ++p) {
      const double sx = mat_at(a, {(size_t)p, 2}), sy = mat_at(a, {(size_t)p, 3});
      x.pos.push_back(mat_at(a, {(size_t)p, 0}));
      x.pos.push_back(mat_at(a, {(size_t)p, 1}));
      x.pos.push_back(sx * sx);
      x.pos.push_back(sy * sy);
    }
    require(!torso_det_dir.empty(), "the position score needs the torso detections");
    char name[64];
    std::snprintf(name, sizeof name, "/pose_est_imgidx%04d.mat", imgidx);
    const auto d = mat_read(torso_det_dir + name);
    const MatArray &bc = mat_find(d, "best_conf");
    const int k = rootidx_det >= 0 ? rootidx_det : root;
    require(bc.dims.size() == 2 && (int)bc.dims[0] > k && bc.dims[1] >= 6, "best_conf: [P][7]");
    x.root_det_x = (double)(int)mat_at(bc, {(size_t)k, 4});  // int root_pos_x
    x.root_det_y = (double)(int)mat_at(bc, {(size_t)k, 5});
  }
  if (!torso_prior_file.empty()) {
    const auto v = mat_read(torso_prior_file);
    const MatArray &a = mat_find(v, "params");
    require(a.dims.size() == 2 && a.dims[1] >= 4, "torso prior params: [1][4]");
    for (size_t j = 0; j < 4; ++j) x.torso.push_back(mat_at(a, {0, j}));
    x.torso_weight = torso_weight;
  }
  return x;
}

namespace {

// One [H][W] MATLAB array (column-major) as a row-major float grid.
void dpm_grid(const MatArray &a, int H, int W, const std::string &what, float *dst) {
  require(!a.is_cell() && a.dims.size() == 2 && (int)a.dims[0] == H && (int)a.dims[1] == W,
          what + ": scoregrid is not [" + std::to_string(H) + "][" + std::to_string(W) + "]");
  for (int y = 0; y < H; ++y)
    for (int xx = 0; xx < W; ++xx) dst[(size_t)y * W + xx] = (float)a.re[y + (size_t)H * xx];
}

std::string dpm_file(const std::string &dir, int imgidx) {
  char name[64];
  std::snprintf(name, sizeof name, "/imgidx_%04d.mat", imgidx + 1);
  return dir + name;
}

// The cell form of loadDPMScoreGrid: a [Rd][1] cell of [H][W] grids.
void dpm_cell(const std::string &path, int Rd, int H, int W, float *dst) {
  const auto v = mat_read(path);
  const MatArray &c = mat_find(v, "scoregrid");
  require(c.is_cell() && c.dims.size() == 2 && (int)c.dims[0] == Rd && c.dims[1] == 1,
          path + ": scoregrid is not a [" + std::to_string(Rd) + "][1] cell");
  for (int r = 0; r < Rd; ++r) dpm_grid(c.cells[r], H, W, path, dst + (size_t)r * H * W);
}

}  // namespace

std::vector<float> loadDetectionMask(const std::string &dir, int imgidx, int S, int H, int W) {
  char name[64];
  std::snprintf(name, sizeof name, "/detection_mask_imgidx%05d.mat", imgidx + 1);
  const std::string path = dir + name;
  const auto v = mat_read(path);
  const MatArray &a = mat_find(v, "detection_mask");
  // mat_load_multi_array keeps MATLAB's dims: element (s, y, x)
  require(!a.is_cell() && a.dims.size() == 3 && (int)a.dims[0] >= S && (int)a.dims[1] == H &&
              (int)a.dims[2] == W,
          path + ": detection_mask is not [>=" + std::to_string(S) + "][" + std::to_string(H) +
              "][" + std::to_string(W) + "]");
  std::vector<float> m((size_t)S * H * W);
  for (int s = 0; s < S; ++s)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x)
        m[((size_t)s * H + y) * W + x] = (float)mat_at(a, {(size_t)s, (size_t)y, (size_t)x});
  return m;
}

void loadDpmScores(ExtraUnaryParams &x, int imgidx, int n_parts, int R, int H, int W,
                   const DpmOptions &o) {
  const size_t HW = (size_t)H * W;
  if (!o.torso_dir.empty()) {
    const std::string path = dpm_file(o.torso_dir, imgidx);
    const auto v = mat_read(path);
    x.dpm_torso.resize(HW);
    dpm_grid(mat_find(v, "scoregrid"), H, W, path, x.dpm_torso.data());
    x.dpm_torso_weight = o.torso_weight;
  }
  auto detect = [&](int p) { return x.is_detect.empty() || x.is_detect[p] != 0; };
  if (o.head && !o.unary_dir.empty()) {
    x.dpm_head_part = n_parts == 22 ? 11 : n_parts == 12 ? 1 : 5;
    require(x.dpm_head_part < n_parts, "DPM head: no head part");
    if (detect(x.dpm_head_part)) {
      x.dpm_head.resize(HW);
      dpm_cell(dpm_file(o.unary_dir + "/head", imgidx), 1, H, W, x.dpm_head.data());
      x.dpm_head_weight = o.head_weight;
    }
  }
  if (o.unary && !o.unary_dir.empty()) {
    const int Rd = o.rot ? R : 1;
    x.dpm_unary.assign((size_t)n_parts * Rd * HW, 0.f);
    for (int p = 0; p < n_parts; ++p) {
      if (!detect(p)) continue;
      char sub[32];
      std::snprintf(sub, sizeof sub, "/pidx_%04d", p);
      dpm_cell(dpm_file(o.unary_dir + sub, imgidx), Rd, H, W, x.dpm_unary.data() + (size_t)p * Rd * HW);
    }
    x.dpm_unary_rot = o.rot ? 1 : 0;
    x.dpm_unary_weight = o.unary_weight;
  }
}

std::string scoreGridFileName(const std::string &dir, int imgidx, int pidx, bool flip) {
  return dir + "/imgidx" + std::to_string(imgidx) + "-pidx" + std::to_string(pidx) + "-o" +
         std::to_string(flip ? 1 : 0) + "-scoregrid.mat";
}

ScoreGridSet loadScoreGrid(const std::string &path) {
  const std::vector<MatArray> vars = mat_read(path);
  const MatArray &cell = mat_find(vars, "cell_scoregrid");
  const MatArray &ti2 = mat_find(vars, "transform_Ti2");
  const MatArray &t2g = mat_find(vars, "transform_T2g");
  require(cell.is_cell() && cell.dims.size() == 2, path + ": cell_scoregrid is not a 2-d cell");
  ScoreGridSet g;
  g.S = (int)cell.dims[0];
  g.R = (int)cell.dims[1];
  for (const MatArray *t : {&ti2, &t2g})
    require(!t->is_cell() && t->dims.size() == 4 && (int)t->dims[0] == g.S &&
                (int)t->dims[1] == g.R && t->dims[2] == 3 && t->dims[3] == 3,
            path + ": transforms are not [scales][rotations][3][3]");
  for (int s = 0; s < g.S; ++s)
    for (int r = 0; r < g.R; ++r) {
      const MatArray &e = cell.cells[(size_t)s + (size_t)g.S * r];  // Fortran order
      require(!e.is_cell() && e.dims.size() == 2, path + ": a score grid is not 2-d");
      const int ny = (int)e.dims[0], nx = (int)e.dims[1];
      std::vector<float> v((size_t)ny * nx);
      for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) v[(size_t)y * nx + x] = (float)e.re[(size_t)y + (size_t)ny * x];
      g.ny.push_back(ny);
      g.nx.push_back(nx);
      g.grid.push_back(std::move(v));
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          // the float arrays become the double matrices of the product
          g.Ti2.push_back((double)(float)mat_at(ti2, {(size_t)s, (size_t)r, (size_t)i, (size_t)j}));
          g.T2g.push_back((double)(float)mat_at(t2g, {(size_t)s, (size_t)r, (size_t)i, (size_t)j}));
        }
    }
  return g;
}

FindObjResult findObjectImageFromScoreGrids(Context &ctx, const PartApp &part_app, bool flip,
                                            const std::vector<Joint> &joints,
                                            const std::vector<ScoreGridSet> &parts, int img_h,
                                            int img_w, bool want_marginals) {
  const pa_exp_param e = part_app.m_exp_param.c();
  const int P = part_app.m_part_conf.part_size();
  const int S = std::max(1, e.num_scale_steps), R = e.num_rotation_steps;
  require((int)parts.size() >= P, "saved score grids for every part");
  const size_t N = (size_t)R * img_h * img_w;
  std::vector<float> lu((size_t)P * S * N);
  for (int p = 0; p < P; ++p) {
    const ScoreGridSet &g = parts[p];
    require(g.S == S && g.R == R, "saved score grids: scale or rotation count differs");
    for (int s = 0; s < S; ++s) {
      // one pa_unary_maps call per (part, scale): the grids of a scale share
      // their size; Tig = prod(Ti2, T2g) per rotation (partapp.cpp:877-880)
      const int ny = g.ny[(size_t)s * R], nx = g.nx[(size_t)s * R];
      std::vector<float> sc((size_t)R * ny * nx);
      std::vector<double> tig((size_t)R * 9);
      for (int r = 0; r < R; ++r) {
        const size_t k = (size_t)s * R + r;
        require(g.ny[k] == ny && g.nx[k] == nx, "saved score grids of one scale differ in size");
        std::memcpy(sc.data() + (size_t)r * ny * nx, g.grid[k].data(), sizeof(float) * ny * nx);
        const double *a = &g.Ti2[k * 9], *b = &g.T2g[k * 9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int q = 0; q < 3; ++q) acc += a[i * 3 + q] * b[q * 3 + j];
            tig[(size_t)r * 9 + i * 3 + j] = acc;
          }
      }
      ctx.check(pa_unary_maps(ctx.get(), sc.data(), 1, R, ny, nx, tig.data(), 0, e.interpolate,
                              img_h, img_w, lu.data() + ((size_t)p * S + s) * N, PA_MEM_HOST));
    }
  }
  applyExtraUnaries(ctx, part_app, lu, img_h, img_w);
  const TreeHolder th(part_app.m_part_conf, part_app.m_part_conf.rootpart_idx, joints);
  const int K = e.roi_save_num_samples > 0 ? e.roi_save_num_samples : 1;
  ImageOut out(P, K, S);
  std::vector<float> marg;
  if (want_marginals) {
    marg.resize((size_t)P * S * N);
    out.o.log_marg = marg.data();
  }
  ctx.check(pa_ps_infer(ctx.get(), &e, &th.t, flip ? 1 : 0, 1, lu.data(), img_h, img_w, &out.o,
                        PA_MEM_HOST));
  FindObjResult r = out.result(P, K);
  if (want_marginals)
    for (size_t k = 0; k < (size_t)P * S; ++k) {
      FloatGrid3 g(R, img_h, img_w);
      std::memcpy(g.data(), marg.data() + k * N, N * sizeof(float));
      r.log_marginals.push_back(std::move(g));
    }
  return r;
}

bool saveResults(const std::string &dir, int imgidx, bool flip, const FindObjResult &r) {
  const size_t P = r.best_conf.size();
  std::vector<float> bc;
  for (const PartHyp &h : r.best_conf) {
    const std::vector<float> v = h.toVect();
    bc.insert(bc.end(), v.begin(), v.end());
  }
  char name[64];
  std::snprintf(name, sizeof name, "/pose_est_imgidx%04d.mat", imgidx);
  if (!mat_save_float(dir + name, "best_conf", {P, 7}, bc.data())) return false;
  for (size_t p = 0; p < r.log_marginals.size(); ++p) {
    const FloatGrid3 &g = r.log_marginals[p];
    const std::string f = dir + "/log_part_posterior_final_imgidx" + std::to_string(imgidx) +
                          "_scaleidx0_o" + std::to_string(flip ? 1 : 0) + "_pidx" +
                          std::to_string(p) + ".mat";
    if (!mat_save_float(f, "log_prob_grid", {g.shape()[0], g.shape()[1], g.shape()[2]}, g.data()))
      return false;
  }
  return true;
}

std::vector<FindObjResult> findObjectDataset(Context &ctx, const PartApp &part_app, bool flip,
                                             const std::vector<std::vector<Joint>> &joints,
                                             const float *desc, int n_images, int ny, int nx,
                                             int dim, const double Tig[9], int H, int W,
                                             bool want_marginals) {
  require(n_images >= 1 && (int)joints.size() == n_images, "one joint set per image");
  const int P = part_app.m_part_conf.part_size();
  const pa_exp_param e = part_app.m_exp_param.c();
  const int K = e.roi_save_num_samples > 0 ? e.roi_save_num_samples : 1;
  std::vector<TreeHolder> holders;
  holders.reserve(n_images);
  std::vector<pa_tree> trees;
  for (int i = 0; i < n_images; ++i) {
    holders.emplace_back(part_app.m_part_conf, part_app.m_part_conf.rootpart_idx, joints[i]);
    trees.push_back(holders.back().t);
  }
  std::vector<ImageOut> outs;
  outs.reserve(n_images);
  std::vector<pa_ps_outputs> o;
  const int R = e.num_rotation_steps;
  const size_t N = (size_t)R * H * W;
  std::vector<std::vector<float>> marg(want_marginals ? n_images : 0);
  for (int i = 0; i < n_images; ++i) {
    outs.emplace_back(P, K);
    o.push_back(outs.back().o);
    if (want_marginals) {
      marg[i].resize((size_t)P * N);
      o.back().log_marg = marg[i].data();
    }
  }
  std::vector<const pa_classifier *> cls;
  for (const AdaBoostClassifier *a : part_app.m_abc) cls.push_back(a->get());
  ctx.check(pa_find_obj_batch(ctx.get(), &e, n_images, trees.data(), flip ? 1 : 0, cls.data(),
                              (int)cls.size(), desc, ny, nx, dim, Tig, 1, H, W, nullptr, o.data(),
                              PA_MEM_HOST));
  std::vector<FindObjResult> res;
  for (int i = 0; i < n_images; ++i) {
    res.push_back(outs[i].result(P, K));
    if (want_marginals)
      for (int p = 0; p < P; ++p) {
        FloatGrid3 g(R, H, W);
        std::memcpy(g.data(), marg[i].data() + (size_t)p * N, N * sizeof(float));
        res.back().log_marginals.push_back(std::move(g));
      }
  }
  return res;
}

// ------------------------------------------------------------------------
// Part configuration and joints of a reference experiment
// ------------------------------------------------------------------------
namespace {

// Tokens of the protobuf text format: names, numbers, quoted strings and the
// punctuation : { } < > ; , (comments run from # to the end of the line).
struct PbTokens {
  std::vector<std::string> t;
  size_t i = 0;
  explicit PbTokens(const std::string &s) {
    size_t k = 0;
    while (k < s.size()) {
      const char c = s[k];
      if (std::isspace((unsigned char)c)) { ++k; continue; }
      if (c == '#') {
        while (k < s.size() && s[k] != '\n') ++k;
        continue;
      }
      if (c == '"' || c == '\'') {
        std::string v(1, '"');
        ++k;
        while (k < s.size() && s[k] != c) {
          if (s[k] == '\\' && k + 1 < s.size()) ++k;
          v += s[k++];
        }
        if (k >= s.size()) throw std::runtime_error("part configuration: unterminated string");
        ++k;
        t.push_back(v);
        continue;
      }
      if (std::strchr(":{}<>;,[]", c)) {
        t.emplace_back(1, c);
        ++k;
        continue;
      }
      const size_t b = k;
      while (k < s.size() && !std::isspace((unsigned char)s[k]) && !std::strchr(":{}<>;,[]#\"'", s[k]))
        ++k;
      t.push_back(s.substr(b, k - b));
    }
  }
  bool done() const { return i >= t.size(); }
  const std::string &peek() const {
    if (done()) throw std::runtime_error("part configuration: unexpected end");
    return t[i];
  }
  std::string next() {
    const std::string &v = peek();
    ++i;
    return v;
  }
  void skip_sep() {
    while (!done() && (t[i] == ";" || t[i] == ",")) ++i;
  }
};

bool pb_is_open(const std::string &s) { return s == "{" || s == "<"; }
bool pb_is_close(const std::string &s) { return s == "}" || s == ">"; }

// A scalar value after "name:"; a list [a, b] is read as its last element.
std::string pb_scalar(PbTokens &tk) {
  if (tk.peek() == "[") {
    tk.next();
    std::string last;
    while (tk.peek() != "]") {
      const std::string v = tk.next();
      if (v != ",") last = v;
    }
    tk.next();
    return last;
  }
  return tk.next();
}

void pb_skip_message(PbTokens &tk) {
  int depth = 1;
  while (depth > 0) {
    const std::string v = tk.next();
    if (pb_is_open(v)) ++depth;
    else if (pb_is_close(v)) --depth;
  }
}

int pb_int(const std::string &v) {
  char *end = nullptr;
  const long x = std::strtol(v.c_str(), &end, 0);
  if (v.empty() || *end) throw std::runtime_error("part configuration: not an integer: " + v);
  return (int)x;
}

bool pb_bool(const std::string &v) {
  if (v == "true" || v == "True" || v == "t" || v == "1") return true;
  if (v == "false" || v == "False" || v == "f" || v == "0") return false;
  throw std::runtime_error("part configuration: not a boolean: " + v);
}

// Fields of one message body up to its closing brace; `on_field` gets
// (name, scalar value) and returns false for a field it does not know.
template <class F>
void pb_fields(PbTokens &tk, F on_field) {
  for (;;) {
    tk.skip_sep();
    if (pb_is_close(tk.peek())) {
      tk.next();
      return;
    }
    const std::string name = tk.next();
    if (tk.peek() == ":") tk.next();
    if (pb_is_open(tk.peek())) {  // nested message of a field we do not read
      tk.next();
      pb_skip_message(tk);
      continue;
    }
    on_field(name, pb_scalar(tk));
  }
}

std::string pb_string(const std::string &v) { return !v.empty() && v[0] == '"' ? v.substr(1) : v; }

}  // namespace

PartConfigFile parsePartConfig(const std::string &text) {
  PbTokens tk(text);
  PartConfigFile pc;
  while (!tk.done()) {
    tk.skip_sep();
    if (tk.done()) break;
    const std::string name = tk.next();
    if (tk.peek() == ":") tk.next();
    if (!pb_is_open(tk.next()))
      throw std::runtime_error("part configuration: expected a message after " + name);
    if (name == "part") {
      PartConfigFile::Part p;
      pb_fields(tk, [&](const std::string &f, const std::string &v) {
        if (f == "part_id") p.part_id = pb_int(v);
        else if (f == "is_root") p.is_root = pb_bool(v);
        else if (f == "is_upright") p.is_upright = pb_bool(v);
        else if (f == "is_detect") p.is_detect = pb_bool(v);
      });
      pc.parts.push_back(p);
    } else if (name == "joint") {
      PartConfigFile::JointDef j;
      pb_fields(tk, [&](const std::string &f, const std::string &v) {
        if (f == "child_idx") j.child_id = pb_int(v);
        else if (f == "parent_idx") j.parent_id = pb_int(v);
        else if (f == "type") j.type = pb_string(v);
        else if (f == "num_joint_types") j.num_joint_types = pb_int(v);
      });
      pc.joints.push_back(j);
    } else {
      pb_skip_message(tk);  // app_group and anything else off this path
    }
  }
  return pc;
}

PartConfig partConfigOf(const PartConfigFile &pc) {
  PartConfig out;
  const int P = (int)pc.parts.size();
  if (P < 1) throw std::runtime_error("part configuration: no parts");
  out.is_upright.assign(P, 0);
  out.rootpart_idx = -1;
  for (int p = 0; p < P; ++p) {
    if (pc.parts[p].part_id != p + 1)
      throw std::runtime_error("part configuration: part ids must be 1..n in order");
    out.is_upright[p] = pc.parts[p].is_upright ? 1 : 0;
    if (pc.parts[p].is_detect && pc.parts[p].is_root) {
      if (out.rootpart_idx != -1) throw std::runtime_error("part configuration: two root parts");
      out.rootpart_idx = p;
    }
  }
  if (out.rootpart_idx < 0) throw std::runtime_error("part configuration: no detected root part");
  return out;
}

std::vector<int> loadJointTypes(const PartConfigFile &pc, const std::string &pred_dir, int imgidx,
                                bool is_test) {
  const size_t J = pc.joints.size();
  std::vector<int> tidx(J, -1);
  if (J == 0 || pc.joints[0].num_joint_types <= 1 || imgidx < 0) return tidx;
  const std::string list = is_test ? "test" : "train";
  const std::string path =
      pred_dir + "/" + list + "list_pred_pwise_imgidx_" + std::to_string(imgidx) + ".mat";
  const std::vector<MatArray> vars = mat_read(path);
  const MatArray &c = mat_find(vars, "clusidx_" + list);
  if (c.numel() < J) throw std::runtime_error(path + ": clusidx_" + list + " is shorter than the joints");
  for (size_t j = 0; j < J; ++j) tidx[j] = (int)c.re[j];
  return tidx;
}

std::vector<Joint> loadJoints(const PartConfigFile &pc, const std::string &spatial_dir,
                              const std::vector<int> &tidx) {
  const int P = (int)pc.parts.size();
  std::vector<Joint> js;
  for (size_t j = 0; j < pc.joints.size(); ++j) {
    const PartConfigFile::JointDef &d = pc.joints[j];
    const int t = j < tidx.size() ? tidx[j] : -1;
    const std::string stem =
        spatial_dir + "/joint_" + std::to_string(d.child_id) + "_" + std::to_string(d.parent_id);
    const std::string gen = stem + ".mat";
    const std::string mix = t > -1 ? stem + "_tidx_" + std::to_string(t) + ".mat" : gen;
    const bool have_mix = std::ifstream(mix).good();
    const std::vector<MatArray> vars = mat_read(have_mix ? mix : gen);
    auto scalar = [&](const char *name) {
      const MatArray &a = mat_find(vars, name);
      if (a.numel() < 1) throw std::runtime_error(gen + ": " + name + " is empty");
      return a.re[0];
    };
    const int type = (int)scalar("type");
    if ((int)scalar("child_idx") != d.child_id || (int)scalar("parent_idx") != d.parent_id)
      throw std::runtime_error(stem + ": child_idx / parent_idx differ from the part configuration");
    Joint J;
    const MatArray &oc = mat_find(vars, "offset_c"), &op = mat_find(vars, "offset_p");
    const MatArray &C = mat_find(vars, "C");
    if (oc.numel() != 2 || op.numel() != 2) throw std::runtime_error(stem + ": offsets must have 2 entries");
    if (C.numel() != 4 || C.dims.size() != 2 || C.dims[0] != 2)
      throw std::runtime_error(stem + ": C must be 2 x 2");
    for (int k = 0; k < 2; ++k) {
      J.offset_c[k] = oc.re[k];
      J.offset_p[k] = op.re[k];
    }
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) J.C[r * 2 + c] = mat_at(C, {(size_t)r, (size_t)c});
    if (type == 2) {  // Joint::ROT_GAUSSIAN
      if (!have_mix) throw std::runtime_error(mix + ": missing mixture component of a rotation joint");
      J.rot_mean = scalar("rot_mean");
      J.rot_sigma = scalar("rot_sigma");
    } else if (type != 1) {  // Joint::POS_GAUSSIAN
      throw std::runtime_error(stem + ": unknown joint type " + std::to_string(type));
    }
    J.child_idx = d.child_id - 1;
    J.parent_idx = d.parent_id - 1;
    if (J.child_idx < 0 || J.child_idx >= P || J.parent_idx < 0 || J.parent_idx >= P)
      throw std::runtime_error(stem + ": part id outside the configuration");
    js.push_back(J);
  }
  if ((int)js.size() != P - 1) throw std::runtime_error("part configuration: need n_parts - 1 joints");
  return js;
}

}  // namespace partapp_gpu
