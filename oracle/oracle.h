/*
 * oracle.h -- C API of the CPU restatement of partapp's inference hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the partapp_gb300
 * package, its CUDA kernels or its C-ABI library) links, loads or calls this
 * code.  Only tests/, __graft_entry__.smoke() and the cpu_baseline / reference
 * arm of bench.py use it, and only as the checker or as the timed CPU
 * baseline.
 *
 * Every function restates one reference function; the reference file:line is
 * cited beside each declaration (paths are relative to the reference tree).
 * Two numeric flavours exist for the PS path:
 *   *_f32  follows the reference's float storage and float arithmetic
 *          (FP32 maps, FP32 filter taps, FP32 dot products, float exp/log
 *          results), with the loop order of the reference;
 *   *_f64  is the same algorithm carried out entirely in double precision
 *          (the "FP64 oracle" the error reports are quoted against).
 *
 * Parity pinning: the reference ships no golden vectors for this path (its
 * code_test.zip is missing), so this oracle is pinned by the analytic
 * known-answer tests in tests/test_oracle_kat.py instead.
 */
#ifndef PARTAPP_ORACLE_H_
#define PARTAPP_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Experiment parameters that the hot path reads from ExpParam
 * (libPartApp/ExpParam.proto:189-195,229,282). */
typedef struct {
  int num_rotation_steps;        /* R */
  float min_part_rotation;       /* degrees, default -180 */
  float max_part_rotation;       /* degrees, default +180 */
  float min_object_scale;        /* default 1 */
  float max_object_scale;        /* default 1 */
  float strip_border_detections; /* fraction of image width, default 0 */
  int max_local_max;             /* roi_save_num_samples, default 1000 */
  int use_pairwise;              /* default 1 */
  int sparse_up;                 /* bIsSparse of the upward messages (computeRootPosteriorRot;
                                    findObjectImageRotJoints passes true, :740) and of
                                    orc_rot_joint_marginal_*; matters for full covariances */
  int num_scale_steps;           /* S, default 1 (0 reads as 1) */
} orc_exp;

/* Tree + joints (libPictStruct/objectdetect.h:54-86, already converted to
 * 0-based part indices and already flipped if needed). */
typedef struct {
  int n_parts;
  int root;                   /* index of the part with is_root && is_detect */
  const int *is_upright;      /* [n_parts] */
  int n_joints;
  const int *child;           /* [n_joints] */
  const int *parent;          /* [n_joints] */
  const double *offset_c;     /* [n_joints][2] parent_pos - child_pos */
  const double *offset_p;     /* [n_joints][2] child_pos - parent_pos */
  const double *C;            /* [n_joints][4] row-major 2x2 covariance */
  const double *rot_mean;     /* [n_joints] radians */
  const double *rot_sigma;    /* [n_joints] radians */
} orc_tree;

/* AdaBoostClassifier::evaluateFeaturePoint (libAdaBoost/AdaBoost.h:131-160)
 * over n_loc dense feature vectors of length D (row-major [n_loc][D]). */
void orc_adaboost_eval(const int32_t *f, const float *p, const float *theta,
                       const float *alpha, int n_stumps, float sum_alpha,
                       const float *desc, int64_t n_loc, int D, int normalize,
                       float *out);

/* sum_alpha as accumulated by operator>> (libAdaBoost/AdaBoost.cc:327-331). */
float orc_sum_alpha(const float *alpha, int n_stumps);

/* computeScoreGrid in FeatureGrid::concatenate ("window") form
 * (libPartDetect/partdetect_test.cpp:344-405, FeatureGrid.cpp:137-181,
 * FeatureGrid.h:71-75, partdetect_aux.cpp:245-249).  cells is
 * [ny][nx][Dc], valid is [ny][nx] (0 = descriptor missing).  Output grid is
 * [ny][nx] with NO_CLASS_VALUE (0) where the window cannot be evaluated. */
void orc_score_grid_window(const int32_t *f, const float *p,
                           const float *theta, const float *alpha,
                           int n_stumps, float sum_alpha, const float *cells,
                           const uint8_t *valid, int ny, int nx, int Dc,
                           int gx, int gy, double grid_step, int normalize,
                           float *out);

/* squeezeScoreGrid (libPartDetect/partdetect_test.cpp:407-466): returns the
 * bounding box of cells != NO_CLASS_VALUE in bbox[4] = {minx, miny, maxx,
 * maxy} and 1 if the reference would crop (maxx > minx && maxy > miny). */
int orc_squeeze_bbox(const float *grid, int ny, int nx, int *bbox);

/* transform_grid_fixed_size (libMultiArray/multi_array_transform.hpp:123-257)
 * for TM_NEAREST (0), TM_BILINEAR (1) and TM_DIRECT (2).  T21 is the 3x3
 * row-major matrix mapping grid_in coordinates to grid_out coordinates. */
void orc_transform_grid(const float *grid_in, int in_h, int in_w,
                        float *grid_out, int out_h, int out_w,
                        const double *T21, float default_value, int method);

/* clip_scores_fill + computeLogGrid (libPictStruct/objectdetect_aux.hpp:42-60,
 * libMultiArray/multi_array_op.hpp:154-167). */
void orc_clip_log(float *grid, int64_t n);

/* get_gaussian_filter (libBoostMath/boost_math.cpp:104-117), unnormalised.
 * Writes 2*ksize+1 taps (ksize = floor(3*sigma+0.5)) and returns their
 * count; out must hold at least that many. */
int orc_gaussian_filter(double sigma, double *out);
/* boost_math::eig2d (libBoostMath/boost_math.cpp:40-99): V row-major 2x2,
 * E = (smallest, largest) eigenvalue. */
void orc_eig2d(const double *M, double *V, double *E);

/* computeRotJointMarginal (libPictStruct/objectdetect_findrot.cpp:292-456). */
int orc_rot_joint_marginal_f32(const orc_exp *e, const float *child,
                               float *parent, int R, int H, int W,
                               const double *offset_c, const double *offset_p,
                               const double *C, double rot_mean,
                               double rot_sigma, double scale);
int orc_rot_joint_marginal_f64(const orc_exp *e, const double *child,
                               double *parent, int R, int H, int W,
                               const double *offset_c, const double *offset_p,
                               const double *C, double rot_mean,
                               double rot_sigma, double scale);

/* computeRootPosteriorRot + computePartMarginals + root rotation
 * marginalisation + findLocalMax (objectdetect_findrot.cpp:73-286,470-727;
 * objectdetect_aux.cpp:193-320).  log_unary is [P][S][R][H][W] after
 * clip_scores_fill + computeLogGrid (the function applies the upright mask
 * and the root border strip itself, as the reference does); S =
 * num_scale_steps, each scale an independent pass at scale_from_index(s).
 *   log_marg   [P][S][R][H][W]  final log marginals (log_part_posterior)
 *   best_conf  [P][7]        PartHyp::toVect of the first-max argmax (last scale)
 *   root_post  [S][H][W]     log root posterior over kept rotations
 *   part_hyps  [P][K][7]     local maxima per part, last scale (K = e->max_local_max)
 *   n_part_hyps [P]
 *   root_hyps  [K][4]        (scale, x, y, score) of root local maxima over [S][H][W]
 *   n_root_hyps [1]
 * Any output pointer may be NULL.  Returns 0 on success. */
int orc_ps_infer_f32(const orc_exp *e, const orc_tree *t, const float *log_unary,
                     int H, int W, float *log_marg, float *best_conf,
                     float *root_post, float *part_hyps, int *n_part_hyps,
                     float *root_hyps, int *n_root_hyps);
int orc_ps_infer_f64(const orc_exp *e, const orc_tree *t,
                     const double *log_unary, int H, int W, double *log_marg,
                     float *best_conf, double *root_post, float *part_hyps,
                     int *n_part_hyps, float *root_hyps, int *n_root_hyps);

/* findLocalMax over a [S][H][W] grid (objectdetect_aux.cpp:193-264).
 * Writes up to max_n entries of (s, x, y, value) to out[max_n][4] and
 * returns their count.  Ties in the top-max_n selection keep enumeration
 * order (the reference's std::sort leaves their order unspecified). */
int orc_find_local_max(const float *grid, int S, int H, int W, int max_n,
                       double *out);


/* AdaBoost classifiers (n_stumps each); the first tree->n_parts of them are
 * the part detectors the tree uses, any further ones are evaluated only. */
typedef struct {
  int n_parts;                /* number of classifiers */
  int n_stumps;               /* stumps per classifier */
  const int32_t *f;           /* [n_parts][n_stumps] feature index */
  const float *p;             /* polarity */
  const float *theta;         /* threshold */
  const float *alpha;         /* weight */
  const float *sum_alpha;     /* [n_parts] */
} orc_models;

/* One image of the --find_obj path with freshly computed scores
 * (objectdetect_aux.cpp:368-403 -> partdetect_dense, partdetect_test.cpp:53-294
 * -> findObjectImageRotJoints, objectdetect_findrot.cpp:729-1058):
 * per (part, rotation) dense AdaBoost score grid [ny][nx] (normalised),
 * mapped to the [H][W] image by Tig (3x3 row-major, grid -> image) with
 * TM_BILINEAR if interpolate else TM_DIRECT, clip_scores_fill,
 * computeLogGrid, then computeRootPosteriorRot.  desc is
 * [R][ny][nx][D].  log_unary (optional, [P][R][H][W]) receives the log
 * unaries before the upright mask.  Other outputs as orc_ps_infer_f32. */
int orc_find_obj_f32(const orc_exp *e, const orc_tree *t, const orc_models *m,
                     const float *desc, int ny, int nx, int D, const double *Tig,
                     int interpolate, int H, int W, float *log_unary,
                     float *log_marg, float *best_conf, float *root_post,
                     float *part_hyps, int *n_part_hyps, float *root_hyps,
                     int *n_root_hyps);

/* The CPU baseline: n_img images spread over n_threads worker threads, one
 * image per thread at a time, each image single-threaded as in the reference
 * (mirrors --distribute, src/apps/partapp/main.cpp:355-400).  desc[i] is
 * image i's [R][ny][nx][D] field; best_conf is [n_img][P][7].  Returns 0. */
int orc_find_obj_batch_f32(const orc_exp *e, const orc_tree *t,
                           const orc_models *m, int n_img,
                           const float *const *desc, int ny, int nx, int D,
                           const double *Tig, int interpolate, int H, int W,
                           float *best_conf, int n_threads);

/* The PS half of the --find_obj path from given score grids, for many
 * images with their own trees (findObjectImageRotJoints after
 * partdetect_dense, objectdetect_findrot.cpp:729-1058): scores[i] is image
 * i's [P][R][ny][nx] normalised AdaBoost grids (the tree's P parts), mapped
 * by Tig, clipped and logged as orc_find_obj_f32 does, then
 * computeRootPosteriorRot with bIsSparse = true.  trees[i] is image i's
 * tree (one topology); best_conf is [n_img][P][7].  Images are spread over
 * n_threads threads, one image per thread at a time.  Returns 0. */
int orc_ps_from_scores_batch_f32(const orc_exp *e, const orc_tree *trees, int n_img,
                                 const float *const *scores, int ny, int nx,
                                 const double *Tig, int interpolate, int H, int W,
                                 float *best_conf, int n_threads);

/* ---- SHAPEv5 shape-context descriptors (desc.cpp) ---------------------- */

/* initPatchMask(21) (libKMA2/descriptor/FeatureDescriptor.cpp:118-137) and
 * precompute_patch_idx (libKMA2/ShapeDescriptor.cpp:42-64): mask [21][21]
 * float, lcpos / lrpos [21][21] log-polar angle / radius bin coordinates. */
void orc_patch_tables(float *mask, double *lcpos, double *lrpos);

/* KMAcomputeShape (ShapeDescriptor.cpp:168-261) of one normalised 21 x 21
 * patch: 96 values (3 radii x 4 angles x 8 orientations), integers in
 * [0, 255], or INT_MIN everywhere for a patch without edges. */
void orc_shape_descriptor(const float *patch, float *vec);

/* FeatureGrid(img_width, img_height, x_axis, y_axis, desc_step, _)
 * (libPartDetect/FeatureGrid.cpp:22-97): rect = {min_proj_x, max_proj_x,
 * min_proj_y, max_proj_y}, nx, ny. */
void orc_feature_grid(int img_w, int img_h, const double *x_axis, const double *y_axis,
                      double desc_step, double *rect, int *nx, int *ny);

/* smooth(image_in, smooth_image, sigma) (libKMA2/gauss_iir/gauss_iir.cpp:
 * 1391-1400): recursive Gaussian along y then x.  h, w >= 5. */
int orc_smooth(const float *in, int h, int w, float sigma, float *out);

/* computeDescriptorGrid with SHAPEv5 (libPartDetect/partdetect_aux.cpp:77-190)
 * on a grayscale image [img_h][img_w]: cells [ny][nx][96] (zero where the
 * descriptor window leaves the image), valid [ny][nx].  For desc_size > 10
 * the patches are sampled from the image smoothed once with sigma =
 * patch_scale.  Returns 0. */
int orc_descriptor_grid(const float *image, int img_h, int img_w, const double *x_axis,
                        const double *y_axis, double desc_step, int desc_size, float *cells,
                        uint8_t *valid);

/* computeDescriptorGrid with a detection mask and a region of interest
 * (partdetect_aux.cpp:77-160): detection_mask [img_h][img_w] or NULL (a
 * position whose mask value, at the truncated image coordinates, is 0 gets
 * no descriptor); roi = {x, y, width, height} as QRect(x, y, width, height)
 * holds it, or NULL for the default QRect(0, 0, img_w - 1, img_h - 1). */
int orc_descriptor_grid_ex(const float *image, int img_h, int img_w, const double *x_axis,
                           const double *y_axis, double desc_step, int desc_size,
                           const float *detection_mask, const int *roi, float *cells,
                           uint8_t *valid);

/* add_image_border2 (libKMA2/ImageContent/ImageContent.cpp:937-999): out is
 * [h + 2b][w + 2b]; returns the border used (b, or min(w, h) - 1). */
int orc_add_border(const float *in, int h, int w, int b, float *out);

/* partdetect_dense for one image at one scale, in-memory path
 * (libPartDetect/partdetect_test.cpp:53-294, as findObjectDataset's
 * force_recompute_scores branch runs it), then clip_scores_fill +
 * computeLogGrid: mirrored border, per rotation the rotated FeatureGrid, its
 * SHAPEv5 descriptors, every classifier's window scores (window_size [n][2],
 * grid_x_count = window_size_x / desc_step + 1), squeezeScoreGrid, TM_DIRECT
 * into the image, for each of the num_scale_steps = S scales (the scale loop,
 * :116).  m->n_parts classifiers; log_unary [n][S][R][h][w]. */
int orc_partdetect(const orc_exp *e, const orc_models *m, const int *window_size,
                   const double *pos_offset, int desc_step, int desc_size, double ratio,
                   const float *image, int h, int w, int flip, float *log_unary);

/* orc_partdetect with the per-scale detection masks of partdetect_dense
 * (partdetect_test.cpp:86-99, 135-146): detection_mask [S][h][w], each scale's
 * mask placed in a zero array the size of the bordered image. */
int orc_partdetect_masked(const orc_exp *e, const orc_models *m, const int *window_size,
                          const double *pos_offset, int desc_step, int desc_size, double ratio,
                          const float *image, int h, int w, int flip,
                          const float *detection_mask, float *log_unary);

/* extra unary terms of findObjectImageRotJoints (objectdetect_findrot.cpp:915-948) */
int orc_extra_unary(const orc_exp *e, int P, int root, float rot_weight, const double *rot_params,
                    float pos_weight, const double *pos_params, double root_det_x,
                    double root_det_y, float torso_weight, const double *torso_prior,
                    const int *is_detect, float *lu, int S, int H, int W);

/* addDPMScore + addLoadDPMScore (torso, head, unary DPM grids) on lu
 * [P][S][R][H][W]; raw grids torso/head [H][W], unary [P][unary_rot ? R : 1]
 * [H][W]; a NULL grid switches its term off. */
/* nms_recursive: suppressed flags of hypotheses sorted by descending score;
 * 2 when they are not sorted. */
int orc_nms_recursive(int n, const float *x, const float *y, const float *scale,
                      const float *score, double train_object_width,
                      double train_object_height, int *nms);

/* libNms: rect_from_hyp (corners rect[4][2]) and the rectangle form of
 * nms_recursive (rects [n][4][2], scores descending; 2 when not sorted). */
void orc_rect_from_hyp(float x, float y, float scale, double reference_height,
                       double reference_width, double *rect);
int orc_nms_rects(int n, const double *rects, const double *scores, double ellipse_size,
                  int *nms);

int orc_dpm_score(const orc_exp *e, int P, int root, float torso_weight, const float *torso,
                  float head_weight, int head_part, const float *head, float unary_weight,
                  int unary_rot, const float *unary, const int *is_detect, float *lu, int S,
                  int H, int W);

#ifdef __cplusplus
}
#endif
#endif
