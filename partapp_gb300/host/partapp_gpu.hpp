// partapp_gpu.hpp -- C++ host layer of partapp_gb300 with the reference's
// call surface for the --find_obj hot path.
//
// The reference's functions take boost::multi_array grids and its own
// ExpParam / PartConfig / Joint / PartHyp types (libPictStruct/objectdetect.h,
// libPartApp).  This header keeps those shapes -- FloatGrid3 in C order
// [rot][y][x], per-part stacks [part][scale], joints as after loadJoints --
// and forwards every call to the C-ABI of include/partapp_gb300.h, so a
// caller of the reference can switch with a type alias.  Errors that the
// reference asserts on throw partapp_gpu::Error here.
#ifndef PARTAPP_GPU_HPP_
#define PARTAPP_GPU_HPP_

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "partapp_gb300.h"

namespace partapp_gpu {

struct Error : std::runtime_error {
  Error(pa_status s, const std::string &what) : std::runtime_error(what), status(s) {}
  pa_status status;
};

// boost::multi_array<float, 3> stand-in (libMultiArray/multi_array_def.h:36):
// contiguous, C order, shape()[0] = rotations, [1] = rows, [2] = columns.
class FloatGrid3 {
 public:
  FloatGrid3() = default;
  FloatGrid3(size_t n0, size_t n1, size_t n2, float fill = 0.f)
      : shape_{n0, n1, n2}, data_(n0 * n1 * n2, fill) {}
  const size_t *shape() const { return shape_; }
  size_t num_elements() const { return data_.size(); }
  float *data() { return data_.data(); }
  const float *data() const { return data_.data(); }
  float &operator()(size_t r, size_t y, size_t x) { return data_[(r * shape_[1] + y) * shape_[2] + x]; }
  float operator()(size_t r, size_t y, size_t x) const {
    return data_[(r * shape_[1] + y) * shape_[2] + x];
  }

 private:
  size_t shape_[3] = {0, 0, 0};
  std::vector<float> data_;
};

// The ExpParam fields the path reads (libPartApp/ExpParam.proto).
struct ExpParam {
  int num_rotation_steps = 48;
  float min_part_rotation = -180.f, max_part_rotation = 180.f;
  float min_object_scale = 1.f, max_object_scale = 1.f;
  float strip_border_detections = 0.f;
  int roi_save_num_samples = 1000;
  bool use_pairwise = true;
  bool interpolate = false;
  int num_scale_steps = 1;  // > 1 only for computeRootPosteriorRot (per-scale unaries)
  pa_exp_param c() const;
};

// PartConfig: which part is the root, which parts are upright.
struct PartConfig {
  int rootpart_idx = 0;
  std::vector<int> is_upright;
  int part_size() const { return (int)is_upright.size(); }
};

// struct Joint (libPictStruct/objectdetect.h:54-86) after loadJoints
// (objectdetect_aux.cpp:54-141): 0-based part indices, radians.
struct Joint {
  int child_idx = -1, parent_idx = -1;
  double offset_c[2] = {0, 0};  // parent_pos - child_pos (pixels)
  double offset_p[2] = {0, 0};  // child_pos - parent_pos (pixels)
  double C[4] = {1, 0, 0, 1};   // row-major 2x2 covariance
  double rot_mean = 0, rot_sigma = 0;
};

// struct PartHyp (objectdetect.h:88-195).
struct PartHyp {
  int m_scaleidx = -1;
  double m_scale = 0;
  int m_rotidx = -1;
  double m_rot = 0;  // degrees
  int m_x = -1, m_y = -1;
  float m_score = -1e6f;
  std::vector<float> toVect() const;  // objectdetect.h:139-159
};

// One GPU context (device + stream + workspace).
class Context {
 public:
  explicit Context(int device = 0);
  ~Context();
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  pa_ctx *get() const { return ctx_; }
  void check(pa_status s) const;  // throws Error with pa_last_error

 private:
  pa_ctx *ctx_ = nullptr;
};

// AdaBoostClassifier (libAdaBoost/AdaBoost.h) on the GPU: loaded from the
// reference's text format (AdaBoost.cc:295-338) or from stump arrays.
class AdaBoostClassifier {
 public:
  AdaBoostClassifier(Context &ctx, const std::string &text);
  AdaBoostClassifier(Context &ctx, int dim, const std::vector<pa_stump> &stumps);
  ~AdaBoostClassifier();
  AdaBoostClassifier(const AdaBoostClassifier &) = delete;
  AdaBoostClassifier &operator=(const AdaBoostClassifier &) = delete;
  const pa_classifier *get() const { return cls_; }
  int dim() const;
  int size() const;
  float sum_alpha() const;

 private:
  Context &ctx_;
  pa_classifier *cls_ = nullptr;
};

// The learned unary (no reference counterpart; pa_unary_net): a convolution
// network over descriptor fields that stands in for the AdaBoost unaries of
// chosen parts.  Device pointers throughout.
class UnaryNet {
 public:
  UnaryNet(Context &ctx, int dim, int n_parts, uint64_t seed = 0) : ctx_(ctx) {
    ctx_.check(pa_unary_net_create(ctx_.get(), dim, n_parts, seed, &net_));
  }
  ~UnaryNet() { pa_unary_net_destroy(ctx_.get(), net_); }
  UnaryNet(const UnaryNet &) = delete;
  UnaryNet &operator=(const UnaryNet &) = delete;
  pa_unary_net *get() const { return net_; }
  std::vector<float> params() const {
    int64_t n = 0;
    ctx_.check(pa_unary_net_get_params(ctx_.get(), net_, nullptr, &n));
    std::vector<float> p((size_t)n);
    ctx_.check(pa_unary_net_get_params(ctx_.get(), net_, p.data(), &n));
    return p;
  }
  void set_params(const std::vector<float> &p) {
    ctx_.check(pa_unary_net_set_params(ctx_.get(), net_, p.data()));
  }
  // One Adam step on the squared error against the log of AdaBoost scores
  // [P][n][ny][nx] of the same fields; returns the loss.
  double train_step(const void *fields, bool fields_bf16, const float *scores, int n, int ny,
                    int nx, const pa_adam_param &opt) {
    double loss = 0.0;
    ctx_.check(pa_unary_net_backward(ctx_.get(), net_, fields, fields_bf16 ? 1 : 0, scores, n, ny,
                                     nx, &loss, nullptr));
    ctx_.check(pa_unary_net_adam(ctx_.get(), net_, &opt));
    return loss;
  }

 private:
  Context &ctx_;
  pa_unary_net *net_ = nullptr;
};

// AbcDetectorParam (libPartDetect/AbcDetectorParam.proto:2-12) fields of the
// dense detector.
struct AbcDetectorParam {
  int desc_step = 4;
  int desc_size = 10;
  double window_desc_step_ratio = 1.0;
};

// PartWindowParam.part(p) (libPartDetect/PartWindowParam.proto:8-12).
struct PartWindow {
  int window_size_x = 0, window_size_y = 0;
  double pos_offset_x = 0, pos_offset_y = 0;
};

// What the reference's PartApp carries for this path.
// The poselet-conditioned extra unary terms of findObjectImageRotJoints
// (objectdetect_findrot.cpp:855-948), with their parameters as the reference's
// loaders leave them (getRotParams, getPosParams, getRootPosDet,
// getTorsoPosPriorParams in objectdetect_icps.cpp).  Empty vectors switch a
// term off.
struct ExtraUnaryParams {
  float rot_weight = 0.f;           // pred_unary_rot_weight
  std::vector<double> rot;          // [P][2]: mean rotation (rad), variance
  float pos_weight = 0.f;           // pred_unary_pos_weight
  std::vector<double> pos;          // [P][4]: mu_x, mu_y, var_x, var_y
  double root_det_x = 0, root_det_y = 0;
  float torso_weight = 0.f;         // torso_pos_prior_weight
  std::vector<double> torso;        // [4]: mu_x, mu_y, var_x, var_y
  std::vector<int> is_detect;       // [P] (empty: every part)
  // DPM score terms, added before the terms above (raw grids; empty: off)
  float dpm_torso_weight = 0.f;     // dpm_torso_weight
  std::vector<float> dpm_torso;     // [H][W]
  float dpm_head_weight = 0.f;      // dpm_head_weight
  int dpm_head_part = 5;
  std::vector<float> dpm_head;      // [H][W]
  float dpm_unary_weight = 0.f;     // dpm_unary_weight
  int dpm_unary_rot = 0;            // do_dpm_rot
  std::vector<float> dpm_unary;     // [P][dpm_unary_rot ? R : 1][H][W]
};

// Where the DPM grids lie and how they are weighted (use_dpm_torso with
// test_dpm_torso_dir, use_dpm_head and use_dpm_unary with test_dpm_unary_dir,
// do_dpm_rot).  An empty directory leaves that term off.
struct DpmOptions {
  std::string torso_dir;
  float torso_weight = 1.f;
  bool head = false;
  float head_weight = 1.f;
  bool unary = false;
  std::string unary_dir;
  float unary_weight = 1.f;
  bool rot = false;
};

// Reads the DPM grids of image imgidx as loadDPMScoreGrid
// (objectdetect_icps.cpp:550-576) finds them: <dir>/imgidx_<NNNN>.mat with
// NNNN = imgidx + 1, variable "scoregrid" -- a plain [H][W] array for the
// torso, a cell of [H][W] arrays, one per DPM rotation, for the head
// (<test_dpm_unary_dir>/head) and the unary grids
// (<test_dpm_unary_dir>/pidx_<NNNN>, NNNN = part index, detected parts only).
// The head part is part 5, 1 with 12 parts, 11 with 22 parts
// (objectdetect_findrot.cpp:893-898).
void loadDpmScores(ExtraUnaryParams &x, int imgidx, int n_parts, int R, int H, int W,
                   const DpmOptions &o);

// The detection masks of image imgidx as partdetect_dense loads them
// (libPartDetect/partdetect_test.cpp:89-99): <dir>/detection_mask_imgidx<NNNNN>.mat
// (NNNNN = imgidx + 1, five digits), variable "detection_mask" [S'][H][W]
// with S' >= S; returns the first S masks as [S][H][W] floats.
std::vector<float> loadDetectionMask(const std::string &dir, int imgidx, int S, int H, int W);

// Reads the reference's prediction files for image imgidx:
//   rot:   <pred_dir>/testlist_params_rot_imgidx<i>.mat, "rot_test" [P][2+]
//          (mean, deviation -> variance = deviation^2), getRotParams :193-226
//   pos:   <pred_dir>/testlist_params_pos_imgidx<i>.mat, "pos_test" [P][4+]
//          (mu_x, mu_y, deviations -> variances), getPosParams :326-364
//   root:  <torso_det_dir>/pose_est_imgidx<NNNN>.mat, "best_conf" row
//          rootidx_det, columns 4, 5 truncated to int, getRootPosDet :283-324
//   torso: <torso_prior_file>, "params" [1][4], getTorsoPosPriorParams :32-45
// An empty directory or file name leaves that term off.
ExtraUnaryParams loadExtraUnaryParams(int imgidx, int n_parts, int root, const std::string &pred_dir,
                                      float rot_weight, float pos_weight,
                                      const std::string &torso_det_dir, int rootidx_det,
                                      const std::string &torso_prior_file, float torso_weight);

// PartConfig (libPartDetect/PartConfig.proto) as the protobuf text format of
// an experiment holds it, reduced to the fields this path reads: part ids
// and the is_root / is_upright / is_detect flags, and the joints between
// part ids (child_idx, parent_idx, type, num_joint_types).  Other fields are
// skipped.
struct PartConfigFile {
  struct Part {
    int part_id = 0;
    bool is_root = false, is_upright = false, is_detect = true;
  };
  struct JointDef {
    int child_id = 0, parent_id = 0;  // part ids (1-based)
    std::string type = "Gaussian";
    int num_joint_types = 1;
  };
  std::vector<Part> parts;
  std::vector<JointDef> joints;
};
PartConfigFile parsePartConfig(const std::string &text);

// The root index and upright flags of a part configuration; part ids must be
// 1..P in order (loadJoints asserts part_id == pidx + 1) and exactly one
// detected part the root (findObjectImageRotJoints, objectdetect_findrot.cpp:783-788).
PartConfig partConfigOf(const PartConfigFile &pc);

// Per-joint mixture component of image imgidx, as loadJoints takes it from
// predictFactors' output (objectdetect_aux.cpp:73-92):
// <pred_dir>/<list>list_pred_pwise_imgidx_<imgidx>.mat, vector "clusidx_<list>"
// with list "test" or "train".  Used only when the configuration's first
// joint has num_joint_types > 1; otherwise every entry is -1.
std::vector<int> loadJointTypes(const PartConfigFile &pc, const std::string &pred_dir, int imgidx,
                                bool is_test = true);

// load_joint for every joint of the configuration (libPictStruct/
// objectdetect_learnparam.cpp:92-180) followed by loadJoints' conversion of
// part ids to indices (objectdetect_aux.cpp:54-141): reads
// <spatial_dir>/joint_<child>_<parent>[_tidx_<t>].mat (the general file when
// the mixture file is missing; a missing mixture file of a rotation joint is
// an error, as the reference asserts), variables type, child_idx,
// parent_idx, offset_c, offset_p, C (2 x 2) and, for ROT_GAUSSIAN (type 2),
// rot_mean and rot_sigma.  The flip of loadJoints is not applied here: the
// pa_* entries apply it from their flip argument.  tidx[j] < 0 (or an empty
// vector) selects the general file.
std::vector<Joint> loadJoints(const PartConfigFile &pc, const std::string &spatial_dir,
                              const std::vector<int> &tidx = {});

struct PartApp {
  ExpParam m_exp_param;
  PartConfig m_part_conf;
  std::vector<Joint> m_joints;                    // loadJoints output
  std::vector<const AdaBoostClassifier *> m_abc;  // part detectors first
  AbcDetectorParam m_abc_param;                   // for detection from images
  std::vector<PartWindow> m_window_param;         // one per classifier in m_abc
  const ExtraUnaryParams *m_extra = nullptr;       // extra unary terms, if any
  // the image's detection masks [S][H][W] (exp_param.detection_masks_dir), if any
  const std::vector<float> *m_detection_mask = nullptr;
};

// computeRotJointMarginal (objectdetect_findrot.cpp:292-456): child ->
// parent frame message.  bIsSparse selects TM_DIRECT for the forward
// rotation of a full covariance's map (bilinear otherwise).
void computeRotJointMarginal(Context &ctx, const ExpParam &exp_param, FloatGrid3 &log_prob_child,
                             FloatGrid3 &log_prob_parent, const double offset_c_10[2],
                             const double offset_p_01[2], const double C[4], double rot_mean,
                             double rot_sigma, double scale, bool bIsSparse);

// computeRootPosteriorRot (objectdetect_findrot.cpp:470-727) including
// computePartMarginals and findLocalMax.  log_part_detections[part][scale]
// are the log unaries (after clip_scores_fill + computeLogGrid); they are
// not modified.  best_part_hyp[part] receives the argmax of the part's
// marginal followed by its local maxima, of the last scale as in the
// reference; root_part_posterior is [nScales][H][W].  If log_marginals is
// given it receives the final log marginals in [part][scale] order
// (index part * nScales + scale); log_z is [scale][part].
void computeRootPosteriorRot(Context &ctx, const PartApp &part_app,
                             std::vector<std::vector<FloatGrid3>> &log_part_detections,
                             FloatGrid3 &root_part_posterior, int rootpart_idx,
                             std::vector<Joint> joints, bool flip, bool bIsSparse, int imgidx,
                             std::vector<std::vector<PartHyp>> &best_part_hyp,
                             bool bSaveMarginals,
                             std::vector<FloatGrid3> *log_marginals = nullptr,
                             std::vector<double> *log_z = nullptr);

// computeScoreGrid (libPartDetect/partdetect_test.cpp:344-405) for every
// classifier over dense window descriptors desc[field][ny][nx][dim]:
// scores[c] = FloatGrid3(n_fields, ny, nx).
void computeScoreGrids(Context &ctx, const std::vector<const AdaBoostClassifier *> &abc,
                       const float *desc, int n_fields, int ny, int nx, int dim,
                       bool bNormalizeBoost, std::vector<FloatGrid3> &scores);

// Result of one image of findObjectImageRotJoints.
struct FindObjResult {
  std::vector<PartHyp> best_conf;                 // argmax per part
  std::vector<std::vector<PartHyp>> part_hyps;    // local maxima per part
  std::vector<std::vector<float>> root_hyps;      // (scale, x, y, score)
  std::vector<double> log_z;                      // FP64 log-partition per part
  std::vector<FloatGrid3> log_marginals;          // [part] final log marginals, if asked for
};

// findObjectImageRotJoints (objectdetect_findrot.cpp:729-1058) with freshly
// computed scores: unaries from descriptors desc[R][ny][nx][dim], grid ->
// image transform Tig (3x3, row-major), PS, marginals, local maxima.
FindObjResult findObjectImageRotJoints(Context &ctx, const PartApp &part_app, bool flip,
                                       const float *desc, int ny, int nx, int dim,
                                       const double Tig[9], int H, int W,
                                       bool want_marginals = false);

// findObjectDataset (objectdetect_aux.cpp:322-406) over a batch of images
// with the same sizes; joints[i] are image i's joints (per-image pairwise).
std::vector<FindObjResult> findObjectDataset(Context &ctx, const PartApp &part_app, bool flip,
                                             const std::vector<std::vector<Joint>> &joints,
                                             const float *desc, int n_images, int ny, int nx,
                                             int dim, const double Tig[9], int H, int W,
                                             bool want_marginals = false);

// partdetect (libPartDetect/partdetect_test.cpp:296-341 -> partdetect_dense)
// on a grey image [img_h][img_w] followed by clip_scores_fill + computeLogGrid:
// log_part_detections[classifier][scale] = FloatGrid3(R, img_h, img_w).
// part_app.m_detection_mask, when set, restricts the descriptor positions.
void partdetect(Context &ctx, const PartApp &part_app, const float *image, int img_h,
                int img_w, bool flip, std::vector<std::vector<FloatGrid3>> &log_part_detections);

// findObjectImageRotJoints with freshly computed detections, the
// force_recompute_scores branch of findObjectDataset (objectdetect_aux.cpp:
// 376-384): partdetect on the image (unflipped, as the reference calls it),
// then computeRootPosteriorRot with bIsSparse = true and the joints
// (as stored; mirrored inside when flip).
FindObjResult findObjectImageFromImage(Context &ctx, const PartApp &part_app, bool flip,
                                       const std::vector<Joint> &joints, const float *image,
                                       int img_h, int img_w, bool want_marginals = false);

// One part's saved score grids as PartApp::loadScoreGrid reads them
// (libPartApp/partapp.cpp:830-903) from
// <dir>/imgidx<i>-pidx<p>-o<flip>-scoregrid.mat (getScoreGridFileName,
// partapp.cpp:792-799): cell_scoregrid[scale][rot] grids [ny][nx] (C order
// here) and transform_Ti2 / transform_T2g [scale][rot][3][3].
struct ScoreGridSet {
  int S = 0, R = 0;
  std::vector<int> ny, nx;                 // per (scale, rot)
  std::vector<std::vector<float>> grid;    // per (scale, rot): [ny][nx]
  std::vector<double> Ti2, T2g;            // [S][R][9], row-major 3x3
};
std::string scoreGridFileName(const std::string &dir, int imgidx, int pidx, bool flip);
ScoreGridSet loadScoreGrid(const std::string &path);

// findObjectImageRotJoints with bLoadScoreGrid = true, the default branch of
// findObjectDataset (objectdetect_aux.cpp:382-390): every part's saved grids
// mapped into the image with Tig = Ti2 * T2g per (scale, rot)
// (loadScoreGrid, TM_BILINEAR if interpolate else TM_DIRECT), clip_scores_fill
// + computeLogGrid, then computeRootPosteriorRot with bIsSparse = true.
FindObjResult findObjectImageFromScoreGrids(Context &ctx, const PartApp &part_app, bool flip,
                                            const std::vector<Joint> &joints,
                                            const std::vector<ScoreGridSet> &parts, int img_h,
                                            int img_w, bool want_marginals = false);

// The reference's result files (objectdetect_findrot.cpp:238-251, 1005-1011):
// pose_est_imgidx<NNNN>.mat with best_conf [P][7], and per part
// log_part_posterior_final_imgidx<i>_scaleidx0_o<flip>_pidx<p>.mat with
// log_prob_grid [R][H][W] when the marginals were asked for.
bool saveResults(const std::string &dir, int imgidx, bool flip, const FindObjResult &r);

}  // namespace partapp_gpu

#endif  // PARTAPP_GPU_HPP_
