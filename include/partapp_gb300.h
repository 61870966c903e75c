/*
 * partapp_gb300.h -- C-ABI of the GB300 implementation of partapp's
 * inference hot path (dense AdaBoost part unaries + rotation-aware
 * pictorial-structures sum-product with marginals).
 *
 * The reference has no plugin/FFI layer: its boundary is the in-process C++
 * call surface of libPartDetect / libPictStruct.  Each entry point below names
 * the reference function(s) it replaces (paths relative to the reference
 * tree).  Conventions:
 *   - every call returns a pa_status and never aborts (the reference reports
 *     errors only through assert()); no C++ exception crosses the boundary
 *     (a failed host allocation is PA_ERR_NOMEM);
 *   - maps use the reference's FloatGrid3 layout, C order [rot][y][x], float;
 *     per-part stacks are [part][rot][y][x];
 *   - buffers are caller-owned; `mem` says whether the data pointers of a call
 *     are device (PA_MEM_DEVICE) or host (PA_MEM_HOST) memory.  Host buffers
 *     are staged through the context's device workspace;
 *   - a context is bound to one device and one CUDA stream; calls on one
 *     context must not run concurrently from several host threads.
 */
#ifndef PARTAPP_GB300_H_
#define PARTAPP_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int pa_status;
#define PA_OK 0
#define PA_ERR_INVALID 1      /* argument the reference would assert on */
#define PA_ERR_UNSUPPORTED 2  /* valid for the reference, not built here */
#define PA_ERR_CUDA 3         /* CUDA runtime error (message in pa_last_error) */
#define PA_ERR_NOMEM 4        /* device or host allocation failed */
#define PA_ERR_NUMERIC 5      /* exp() overflow: the reference asserts here */
#define PA_ERR_TIMEOUT 6      /* a bounded device-side wait ran out (pa_find_obj_queue) */

#define PA_MEM_DEVICE 0
#define PA_MEM_HOST 1

#define PA_NO_CLASS_VALUE 0.0f /* libPartDetect/partdetect.h:45 */
#define PA_LOG_ZERO (-1e6f)    /* libBoostMath/boost_math.h:23 */

typedef struct pa_ctx pa_ctx;
typedef struct pa_classifier pa_classifier;

/* ---------------------------------------------------------------- context */

/* Creates a context on `device` with its own non-blocking stream. */
pa_status pa_ctx_create(int device, pa_ctx **out);
pa_status pa_ctx_destroy(pa_ctx *ctx);
/* Makes the context issue its work on `stream` (a cudaStream_t).  Device
 * inputs are read, and device outputs written, in the order of this stream:
 * inputs produced on another stream must be complete there first (set the
 * producing stream here, or make this stream wait on an event).  Calls that
 * return host results return after their work on the stream has finished. */
pa_status pa_ctx_set_stream(pa_ctx *ctx, void *stream);
pa_status pa_ctx_synchronize(pa_ctx *ctx);
/* No counterpart in the reference.  Arithmetic of the spatial Gaussian of
 * diagonal-covariance messages in pa_ps_infer / pa_find_obj*:
 *   PA_MSG_FP32        (default) FP32 shared-memory filters, the reference's
 *                      arithmetic (parity as documented for each entry);
 *   PA_MSG_BF16_TENSOR banded-Toeplitz BF16 products with FP32 accumulation
 *                      on the tensor cores, for large grids (needs H % 8 == 0,
 *                      else the FP32 filters run); its error against FP64 is
 *                      larger than the FP32 path's and is reported by the tests.
 * pa_rot_joint_marginal always uses FP32. */
#define PA_MSG_FP32 0
#define PA_MSG_BF16_TENSOR 1
pa_status pa_ctx_set_message_math(pa_ctx *ctx, int mode);
/* Message of the last failing call on this context (never NULL). */
const char *pa_last_error(const pa_ctx *ctx);
const char *pa_status_string(pa_status s);
/* Number of kernels this context has launched so far. */
uint64_t pa_ctx_kernel_launches(const pa_ctx *ctx);
/* Per-kernel device timing, the GPU counterpart of the reference's
 * get_runtime() prints (objectdetect_findrot.cpp:52-57, 995-998): while
 * enabled, every launch is bracketed by CUDA events on the context's stream
 * and the elapsed times are accumulated per kernel at each call's
 * synchronisation point.  pa_ctx_timing_count snapshots the kernel names;
 * pa_ctx_timing_get reads entry i of that snapshot. */
pa_status pa_ctx_enable_timing(pa_ctx *ctx, int on);
pa_status pa_ctx_timing_reset(pa_ctx *ctx);
int pa_ctx_timing_count(pa_ctx *ctx);
pa_status pa_ctx_timing_get(pa_ctx *ctx, int i, const char **name, double *total_ms,
                            uint64_t *launches);

/* ------------------------------------------------------ experiment params */

/* The ExpParam fields the path reads (libPartApp/ExpParam.proto:160,
 * 189-195, 229, 282; defaults in brackets). */
typedef struct {
  int num_rotation_steps;        /* R [48] */
  float min_part_rotation;       /* degrees [-180] */
  float max_part_rotation;       /* degrees [180] */
  float min_object_scale;        /* [1] */
  float max_object_scale;        /* [1] */
  float strip_border_detections; /* fraction of the width [0] */
  int roi_save_num_samples;      /* local maxima kept per part [1000], <= 2048 */
  int use_pairwise;              /* [1] */
  int interpolate;               /* grid->image TM_BILINEAR if 1, else TM_DIRECT [0] */
  int num_scale_steps;           /* S [1]; 0 reads as 1.  S > 1 needs min < max object
                                    scale and is taken by pa_ps_infer (the pa_find_obj*
                                    entries score one scale of descriptors) */
} pa_exp_param;

void pa_exp_param_default(pa_exp_param *p);

/* ------------------------------------------------------ AdaBoost unaries */

/* One decision stump: DecisionStump (libAdaBoost/AdaBoost.h:30-38) without
 * the training-only fields. */
typedef struct {
  int32_t f;   /* feature index */
  float p;     /* polarity */
  float theta; /* threshold */
  float alpha; /* weight */
} pa_stump;

/* Uploads a classifier; sum_alpha is accumulated in stump order as
 * operator>> does (libAdaBoost/AdaBoost.cc:311-338). */
pa_status pa_classifier_create(pa_ctx *ctx, int dim, const pa_stump *stumps,
                               int n_stumps, pa_classifier **out);
/* Parses the text model format of AdaBoostClassifier::loadClassifier
 * (AdaBoost.cc:295-338): "D\n ns\n (f p alpha J_wse theta)*ns". */
pa_status pa_classifier_parse(pa_ctx *ctx, const char *text, size_t len,
                              pa_classifier **out);
pa_status pa_classifier_destroy(pa_ctx *ctx, pa_classifier *cls);
pa_status pa_classifier_info(const pa_classifier *cls, int *dim, int *n_stumps,
                             float *sum_alpha);

/* Dense part detection: score[p][k][iy][ix] =
 * AdaBoostClassifier::evaluateFeaturePoint(desc[k][iy][ix][:], normalize)
 * for every location of every field k (AdaBoost.h:131-160 called from
 * computeScoreGrid, libPartDetect/partdetect_test.cpp:366-377).  Each
 * location holds its complete dim-long window vector.  Decisions and the
 * float sum follow the reference's stump order bit for bit.
 *   desc    [n_fields][ny][nx][dim]
 *   scores  [n_parts][n_fields][ny][nx] */
pa_status pa_score_grids(pa_ctx *ctx, const pa_classifier *const *cls, int n_parts,
                         const float *desc, int n_fields, int ny, int nx, int dim,
                         int normalize, float *scores, int mem);

/* ------------------------------------------------ shape-context descriptors */

/* FeatureGrid(img_width, img_height, x_axis, y_axis, desc_step, desc_size)
 * (libPartDetect/FeatureGrid.cpp:22-97): size of the grid whose axes are
 * x_axis / y_axis (partdetect_test.cpp:171-185 uses (cos r, sin r) and
 * (-sin r, cos r), x_axis negated for a flipped image) and that covers the
 * rotated image at desc_step pixels.  Host only. */
pa_status pa_feature_grid_size(int img_w, int img_h, const double *x_axis, const double *y_axis,
                               double desc_step, int *nx, int *ny);

/* computeDescriptorGrid(image, grid, "SHAPEv5", no detection mask, whole
 * image) (libPartDetect/partdetect_aux.cpp:77-190) with libKMA2's SHAPEv5
 * descriptor (ShapeDescriptor.cpp:168-261): for every grid position inside
 * the image by desc_size + 1 pixels, a 21 x 21 patch resampled along the
 * axes, normalised, Canny edges (5, 15), a 3 x 4 log-polar x 8 orientation
 * histogram, normalised, clipped at 0.2, renormalised, quantised to
 * integers (int)(512 v) <= 255.  A patch without edges gives INT_MIN in all
 * 96 entries, as the reference's float -> int conversion does on x86-64.
 *   image [img_h][img_w] grey levels; cells [ny][nx][96]; valid [ny][nx]
 *   (0: position outside, its cell zero).  For desc_size > 10 (patch scale
 *   (2 desc_size + 1) / 21 > 1) the patches are sampled from the image
 *   smoothed once by libKMA2's recursive Gaussian (gauss_iir.cpp:1391-1400)
 *   with sigma = patch scale, as the reference does.  The cells feed
 *   pa_score_grids_window. */
pa_status pa_descriptor_grid(pa_ctx *ctx, const float *image, int img_h, int img_w,
                             const double *x_axis, const double *y_axis, double desc_step,
                             int desc_size, float *cells, uint8_t *valid, int mem);

/* computeDescriptorGrid(image, grid, "SHAPEv5", detection_mask, roi)
 * (libPartDetect/partdetect_aux.cpp:77-160; the detection-mask and ROI
 * overloads of partdetect.h:137-141): pa_descriptor_grid, except that a
 * position inside the image also gets no descriptor (valid 0, cell zero)
 *   - when detection_mask [img_h][img_w] (same memory as image; NULL: none)
 *     is 0 at the position's truncated image coordinates, or
 *   - when it lies outside roi = {x, y, width, height} (a host array), the
 *     rectangle QRect(x, y, width, height) spans (inclusive right edge
 *     x + width - 1).  Only a mask value equal to 0 removes a position
 *     (NaN does not, as in the reference's == 0 test).
 *     NULL stands for the default QRect(0, 0, img_w - 1, img_h - 1) of the
 *     reference's other overloads, which excludes the last column and row:
 *     with desc_size = 0 that removes positions past img_w - 2 / img_h - 2;
 *     pa_descriptor_grid applies the same default. */
pa_status pa_descriptor_grid_masked(pa_ctx *ctx, const float *image, int img_h, int img_w,
                                    const double *x_axis, const double *y_axis,
                                    double desc_step, int desc_size,
                                    const float *detection_mask, const int *roi, float *cells,
                                    uint8_t *valid, int mem);

/* AbcDetectorParam fields of the dense part detector
 * (libPartDetect/AbcDetectorParam.proto:2-12). */
typedef struct {
  int desc_step;                 /* pixels between descriptors */
  int desc_size;                 /* descriptor radius in pixels */
  double window_desc_step_ratio; /* (0, 1]: window_step = ratio * desc_step (>= 1) */
} pa_abc_param;

/* PartWindowParam.part(p) fields a part detector's window uses
 * (libPartDetect/PartWindowParam.proto:8-12): window size in pixels and the
 * offset of the part position from the window's grid origin. */
typedef struct {
  int window_size_x, window_size_y;
  double pos_offset_x, pos_offset_y;
} pa_part_window;

/* partdetect_dense (libPartDetect/partdetect_test.cpp:53-294) for one image
 * and the in-memory path of findObjectDataset (force_recompute_scores,
 * objectdetect_aux.cpp:376-384) up to the log unaries findObjectImageRotJoints
 * builds (objectdetect_findrot.cpp:834-845): the image gets the mirrored
 * border of add_image_border2 (ceil(desc_size + max_part_diag / 2) pixels);
 * per rotation of `ep` the rotated FeatureGrid (step window_step), its SHAPEv5
 * descriptor grid, every classifier's window scores (computeScoreGrid with
 * bSqueeze and normalised votes: grid_x_count = window_size_x / desc_step +
 * 1, likewise in y; grid_step = desc_step / window_step), the squeeze to the
 * non-empty box, the TM_DIRECT map into the image by Tig = (Ti_ei Ti2)(T2g
 * Tg4) (where cells share a pixel, window steps <= sqrt 2 px, the last one
 * in the reference's x-outer, y-inner loop wins), then clip_scores_fill +
 * computeLogGrid.  Every one of the
 * num_scale_steps = S scales has its own descriptor step and size
 * (scale * desc_step, round(scale * desc_size)), border and grids (the scale
 * loop, :116); the result feeds pa_ps_infer unchanged.  `flip` negates the
 * grid's x axis (partdetect_test.cpp:181-184; the --find_obj path itself
 * passes 0).  Classifier c needs dim = grid_x_count * grid_y_count * 96.
 *   image      [img_h][img_w] grey levels
 *   log_unary  [n_cls][S][R][img_h][img_w] */
pa_status pa_partdetect(pa_ctx *ctx, const pa_exp_param *ep, const float *image, int img_h,
                        int img_w, int flip, const pa_classifier *const *cls, int n_cls,
                        const pa_part_window *windows, const pa_abc_param *abc,
                        float *log_unary, int mem);

/* pa_partdetect with the detection masks of partdetect_dense
 * (partdetect_test.cpp:86-99: exp_param.detection_masks_dir's per-image
 * FloatGrid3 "detection_mask"): detection_mask [S][img_h][img_w] (same
 * memory as image), one mask per scale.  Each scale's mask is read as if
 * placed in a zero array the size of the bordered image (:135-146), so a
 * descriptor position in the mirrored border, or where the mask is 0, gets
 * no descriptor; windows touching one score NO_CLASS_VALUE, and a grid with
 * no scored window is not squeezed (:436-449).  NULL: pa_partdetect. */
pa_status pa_partdetect_masked(pa_ctx *ctx, const pa_exp_param *ep, const float *image,
                               int img_h, int img_w, int flip, const pa_classifier *const *cls,
                               int n_cls, const pa_part_window *windows,
                               const pa_abc_param *abc, const float *detection_mask,
                               float *log_unary, int mem);

/* computeScoreGrid over a grid of per-cell descriptors: each window vector is
 * the reverse-order concatenation of gx*gy cell descriptors taken every
 * round(k*grid_step) cells (FeatureGrid::concatenate,
 * libPartDetect/FeatureGrid.cpp:137-181); windows past last_valid_grid_pos
 * (FeatureGrid.h:71-75) or touching a cell with valid == 0 get
 * NO_CLASS_VALUE.  dim of every classifier must be gx*gy*dc.
 *   cells   [n_fields][ny][nx][dc], valid [n_fields][ny][nx] (uint8)
 *   scores  [n_parts][n_fields][ny][nx] */
pa_status pa_score_grids_window(pa_ctx *ctx, const pa_classifier *const *cls,
                                int n_parts, const float *cells, const uint8_t *valid,
                                int n_fields, int ny, int nx, int dc, int gx, int gy,
                                double grid_step, int normalize, float *scores, int mem);

/* Score grids -> log unary maps: transform_grid_fixed_size(grid -> image,
 * Tig, NO_CLASS_VALUE, TM_BILINEAR or TM_DIRECT) as in PartApp::loadScoreGrid
 * (libPartApp/partapp.cpp:876-899) / partdetect_dense
 * (partdetect_test.cpp:268-292), then clip_scores_fill + computeLogGrid
 * (objectdetect_findrot.cpp:834-845).  Tig is [n_parts][R][9] (row-major
 * 3x3, grid -> image), or one shared [9] matrix if tig_shared.  With
 * interpolate = 0 (TM_DIRECT) cells that round to one pixel leave the value
 * of the last of them in the reference's loop (x1 outer, y1 inner).
 *   scores    [n_parts][R][ny][nx]
 *   log_unary [n_parts][R][H][W] */
pa_status pa_unary_maps(pa_ctx *ctx, const float *scores, int n_parts, int R, int ny,
                        int nx, const double *Tig, int tig_shared, int interpolate, int H,
                        int W, float *log_unary, int mem);

/* -------------------------------------------------- pictorial structures */

/* Tree and joints in host memory: struct Joint
 * (libPictStruct/objectdetect.h:54-86) after loadJoints
 * (objectdetect_aux.cpp:54-141), i.e. 0-based part indices, radians. */
typedef struct {
  int n_parts;
  int root;                /* the part with is_root && is_detect */
  const int *is_upright;   /* [n_parts] PartDef.is_upright */
  int n_joints;            /* must be n_parts - 1 */
  const int *child;        /* [n_joints] */
  const int *parent;       /* [n_joints] */
  const double *offset_c;  /* [n_joints][2] */
  const double *offset_p;  /* [n_joints][2] */
  const double *C;         /* [n_joints][4] row-major 2x2 covariance */
  const double *rot_mean;  /* [n_joints] radians */
  const double *rot_sigma; /* [n_joints] radians */
} pa_tree;

/* PartHyp::toVect order (objectdetect.h:139-159). */
typedef struct {
  float scaleidx, scale, rotidx, rot, x, y, score;
} pa_part_hyp;

/* Outputs of one image.  Every pointer may be NULL.  Map outputs live in the
 * call's `mem` space, the rest in host memory.  S = num_scale_steps (1 for
 * the pa_find_obj* entries).
 *   log_marg     [P][S][R][H][W] final log marginals (log_part_posterior)
 *   root_post    [S][H][W]    log root posterior over the kept rotations
 *   best         [P]          first-maximum argmax of each marginal (of the
 *                             last scale; scaleidx = S - 1)
 *   part_hyps    [P][roi_save_num_samples] local maxima (of the last scale),
 *                             n_part_hyps [P]
 *   root_hyps    [1000][4]    (scale, x, y, score) over [S][H][W], n_root_hyps [1]
 *   log_z        [S][P]       FP64 log(sum exp(log_marg[p])) per part; the
 *                             root's entry is the log-partition function
 *   msg_max      [S][2*(P-1)] FP64 copy of the per-message normaliser in_M:
 *                             [j] upward message over joint j, [P-1+j] the
 *                             downward message over joint j */
typedef struct {
  float *log_marg;
  float *root_post;
  pa_part_hyp *best;
  pa_part_hyp *part_hyps;
  int *n_part_hyps;
  float *root_hyps;
  int *n_root_hyps;
  double *log_z;
  double *msg_max;
} pa_ps_outputs;

/* computeRootPosteriorRot + computePartMarginals + root rotation
 * marginalisation + findLocalMax (libPictStruct/objectdetect_findrot.cpp:
 * 73-286, 470-727; objectdetect_aux.cpp:193-320) on log unaries that went
 * through clip_scores_fill + computeLogGrid.  The upright mask and the root
 * border strip are applied inside, as in the reference.  `flip` applies
 * loadJoints' mirroring (objectdetect_aux.cpp:98-116) to the joints.
 * Supported trees: the root may have any number of children, every other
 * part at most one (the reference asserts this at :210); PA_ERR_UNSUPPORTED
 * otherwise.  Covariances must be symmetric positive definite: diagonal ones
 * take gaussFilterDiag2d, others gaussFilter2dOffset (rotation into the
 * eigenbasis, libMultiArray/multi_array_filter.hpp:335-369).  is_sparse is
 * computeRootPosteriorRot's bIsSparse: the upward messages rotate a full
 * covariance's map into its eigenbasis by TM_DIRECT when set (bilinear
 * otherwise); the downward messages are always dense (:174-179, 224-229).
 * pa_find_obj* pass is_sparse = 1, as findObjectImageRotJoints does (:740).
 * With num_scale_steps = S > 1 every scale is an independent pass with the
 * joints at scale_from_index(s) (the scale loop :503-678); best and
 * part_hyps come from the last scale, as computePartMarginals leaves them,
 * and the root maxima are taken over the [S][H][W] posterior with scale
 * neighbours (findLocalMax, objectdetect_aux.cpp:193-236).  Without pairwise
 * terms the maxima are those of scale 0 (getMaxStates, :73-110).
 *   log_unary [P][S][R][H][W] */
pa_status pa_ps_infer(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                      int is_sparse, const float *log_unary, int H, int W,
                      const pa_ps_outputs *out, int mem);

/* computeRotJointMarginal (objectdetect_findrot.cpp:292-456): one message
 * child -> parent frame; is_sparse = bIsSparse (TM_DIRECT forward rotation
 * of a full covariance).  child, parent [R][H][W]; C as in pa_ps_infer. */
pa_status pa_rot_joint_marginal(pa_ctx *ctx, const pa_exp_param *ep, const float *child,
                                float *parent, int R, int H, int W, const double *offset_c,
                                const double *offset_p, const double *C, double rot_mean,
                                double rot_sigma, double scale, int is_sparse, int mem);

/* No counterpart in the reference.  pa_rot_joint_marginal for callers that
 * cannot allocate device memory on their call path (a host application that
 * keeps all device memory in its own pool, or a loop that must not hit
 * cudaMalloc/cudaFree because they can synchronise the device).  It allocates
 * nothing: its scratch is one static device array of fixed size in the
 * library, held by every GPU that loads it.  child and parent are device
 * pointers; `stream` is a cudaStream_t (NULL: the legacy default stream) and
 * the call returns after the work on it has finished.
 * Limits: R*H*W <= PA_NOALLOC_MAX_CELLS, R <= 64, H + W <= 4096, at most
 * 1024 spatial taps per axis; larger sizes return PA_ERR_NOMEM.  C must be
 * diagonal (PA_ERR_UNSUPPORTED otherwise: the rotated-grid path of a full
 * covariance needs scratch sized by the rotation).
 * Calls share the array: calls whose GPU work overlaps race.  Every call
 * looks up the array's address on the current device (so it stays right
 * after a cudaDeviceReset); child and parent must be memory of that device
 * (PA_ERR_INVALID otherwise).  The first call on a device may load the
 * library's module there: make it before any stream capture. */
#define PA_NOALLOC_MAX_CELLS 2097152
pa_status pa_rot_joint_marginal_noalloc(const pa_exp_param *ep, const float *child,
                                        float *parent, int R, int H, int W,
                                        const double *offset_c, const double *offset_p,
                                        const double *C, double rot_mean, double rot_sigma,
                                        double scale, void *stream);

/* ---------------------------------------------------- building blocks */

/* No counterpart in the reference.  The BF16 tensor-core GEMM the
 * large-grid message path is built on, exposed so that it can be checked on
 * its own: C[M][N] = A[M][K] * B[N][K]^T with bf16 operands (K contiguous,
 * row strides lda, ldb in elements, multiples of 8, 16-byte aligned bases)
 * and fp32 accumulation and output (row stride ldc).  band >= 0 declares A
 * banded (A[m][k] = 0 for |k - m| > band: only the band is read); band < 0:
 * dense.  Device pointers; returns after the product is complete. */
pa_status pa_gemm_bf16(pa_ctx *ctx, const void *A, int64_t lda, const void *B, int64_t ldb,
                       float *C, int64_t ldc, int M, int N, int K, int band);

/* ---------------------------------------------------- the --find_obj path */

/* One image of `partapp --find_obj` with freshly computed scores
 * (findObjectDataset, objectdetect_aux.cpp:368-403 -> partdetect_dense ->
 * findObjectImageRotJoints, objectdetect_findrot.cpp:729-1058):
 * pa_score_grids + pa_unary_maps + pa_ps_infer in one call.  All n_cls
 * classifiers are evaluated (partdetect_dense scores every classifier it
 * loads); the first tree->n_parts of them are the part detectors the tree
 * uses.
 *   desc       [R][ny][nx][dim]
 *   Tig        as pa_unary_maps for the first n_parts classifiers
 *   scores_out [n_cls][R][ny][nx] score grids (may be NULL), in `mem`
 * One scale (num_scale_steps <= 1; several: pa_find_obj_scales). */
pa_status pa_find_obj(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                      const pa_classifier *const *cls, int n_cls, const float *desc, int ny,
                      int nx, int dim, const double *Tig, int tig_shared, int H, int W,
                      float *scores_out, const pa_ps_outputs *out, int mem);

/* One scale's descriptor fields for pa_find_obj_scales. */
typedef struct {
  const float *desc;  /* [R][ny][nx][dim], in the call's `mem` space */
  int ny, nx, dim;
  const double *Tig;  /* as pa_find_obj: [n_parts][R][9], or one [9] if tig_shared */
  int tig_shared;
} pa_scale_fields;

/* pa_find_obj at num_scale_steps = S scales (the scale loop of
 * partdetect_dense, partdetect_test.cpp:116, and of computeRootPosteriorRot,
 * objectdetect_findrot.cpp:503-678): fields[s] holds scale s's descriptors
 * (their grid size and Tig differ per scale); each scale's normalised score
 * grids of the first tree->n_parts classifiers go through pa_unary_maps into
 * the [P][S][R][H][W] log unaries, then pa_ps_infer with bIsSparse.  Outputs
 * as pa_ps_infer's for S scales; with S = 1 the results equal pa_find_obj's.
 * Keeps one device block of P * (S + 1) * R * H * W floats (plus one scale's
 * scores) in the context between calls. */
pa_status pa_find_obj_scales(pa_ctx *ctx, const pa_exp_param *ep, const pa_tree *tree, int flip,
                             const pa_classifier *const *cls, int n_cls,
                             const pa_scale_fields *fields, int H, int W,
                             const pa_ps_outputs *out, int mem);

/* A batch of images sharing sizes and classifiers, each with its own tree
 * parameters (the per-image pairwise terms of poselet-conditioned models),
 * processed together: one launch per pipeline phase covers every image.
 *   desc       [n_images][R][ny][nx][dim] in `mem`
 *   trees      [n_images] host structs (same topology, own joint parameters)
 *   scores_out [n_cls][n_images*R][ny][nx] (may be NULL), in `mem`
 *   out        [n_images] output sets as pa_find_obj */
pa_status pa_find_obj_batch(pa_ctx *ctx, const pa_exp_param *ep, int n_images,
                            const pa_tree *trees, int flip, const pa_classifier *const *cls,
                            int n_cls, const float *desc, int ny, int nx, int dim,
                            const double *Tig, int tig_shared, int H, int W, float *scores_out,
                            const pa_ps_outputs *out, int mem);

/* One image of pa_find_obj_multi: its own experiment parameters (rotation
 * count), tree, sizes, transform and outputs. */
typedef struct {
  const pa_exp_param *ep;
  const pa_tree *tree;
  int flip;
  const float *desc;      /* [R][ny][nx][dim] in the call's `mem` space */
  int ny, nx, dim;
  const double *Tig;      /* as pa_find_obj */
  int tig_shared;
  int H, W;
  const pa_ps_outputs *out;
} pa_image;

/* The image loop of findObjectDataset (objectdetect_aux.cpp:322-406) over
 * images of uneven sizes and rotation counts: images that share parameters,
 * sizes and a shared Tig run together as one batch (one launch per pipeline
 * phase for all of them, descriptors read where they lie), the groups one
 * after another on the context's stream.  Results equal pa_find_obj per
 * image. */
pa_status pa_find_obj_multi(pa_ctx *ctx, int n_images, const pa_image *imgs,
                            const pa_classifier *const *cls, int n_cls, int mem);

/* ------------------------------------------------- extra unary terms */

/* The poselet-conditioned terms findObjectImageRotJoints adds to the log
 * detections before computeRootPosteriorRot
 * (libPictStruct/objectdetect_findrot.cpp:915-948), in that order:
 *   rotation score  getRotScoreGrid + addExtraUnary (objectdetect_icps.cpp:
 *                   228-281, 524-547): every detected part p and rotation r
 *                   gets + rot_weight * log(max(exp(-(rot_r - mu)^2 / (2 var)), 1e-4))
 *   position score  getPosScoreGrid + addExtraUnary (:366-448): every detected
 *                   part but the root gets, per pixel (x, y),
 *                   + pos_weight * log(max(gx * gy, 1e-4)) with
 *                   gx = exp(-(x - root_det_x - mu_x)^2 / (2 var_x)), gy alike
 *   torso prior     setTorsoPosPrior (:137-191): the root part gets
 *                   + log(max(torso_weight * gx * gy, 1e-4)) with
 *                   gx = exp(-(W/2 - x - mu_x)^2 / (2 var_x)), gy alike
 * with the reference's float/double typing.  Parameters as the reference's
 * loaders leave them (getRotParams: variance = squared deviation;
 * getPosParams; getRootPosDet; getTorsoPosPriorParams).  A NULL parameter
 * array switches its term off.
 *   log_unary [n_parts][S][R][H][W] (S = num_scale_steps), updated in place */
typedef struct {
  float rot_weight;            /* pred_unary_rot_weight */
  const double *rot_params;    /* [n_parts][2]: mean rotation (radians), variance */
  float pos_weight;            /* pred_unary_pos_weight */
  const double *pos_params;    /* [n_parts][4]: mu_x, mu_y, var_x, var_y (pixels) */
  double root_det_x, root_det_y;  /* rootpos_det: the root detection (pixels) */
  float torso_weight;          /* torso_pos_prior_weight */
  const double *torso_prior;   /* [4]: mu_x, mu_y, var_x, var_y */
  const int *is_detect;        /* [n_parts] PartDef::is_detect flags, or NULL: all */
} pa_extra_unary;

pa_status pa_add_extra_unaries(pa_ctx *ctx, const pa_exp_param *ep, const pa_extra_unary *ex,
                               int n_parts, int root, float *log_unary, int H, int W, int mem);

/* The DPM score terms findObjectImageRotJoints adds to the log detections
 * before the extra unary terms above (libPictStruct/objectdetect_findrot.cpp:
 * 883-914), in that order:
 *   torso  addDPMScore (objectdetect_icps.cpp:488-522) on the root part, every
 *          scale and rotation: + torso_weight * L(x, y) with L the torso grid
 *          after computeLogGrid (0 -> LOG_ZERO = -1e6, else log), in float
 *   head   addLoadDPMScore (:445-486) on part head_part (skipped unless
 *          detected): + (v > 1e-4 ? head_weight * log(v) : log(1e-4)), v the
 *          grid value, the conditional in double
 *   unary  addLoadDPMScore on every detected part with its own grid, per
 *          rotation (unary_rot = 1, do_dpm_rot) or one for all rotations
 * Grids hold the raw (not logged) scores loadDPMScoreGrid (:550-576) reads:
 * torso and head [H][W], unary [n_parts][unary_rot ? R : 1][H][W].  A NULL
 * grid switches its term off.  `mem` tells where log_unary and the grids lie.
 * A torso score below 0 (or NaN) is PA_ERR_INVALID, as computeLogGrid asserts
 * data >= 0; log_unary is then undefined.
 *   log_unary [n_parts][S][R][H][W] (S = num_scale_steps), updated in place */
typedef struct {
  float torso_weight;          /* dpm_torso_weight */
  const float *torso;          /* [H][W] torso DPM scores, or NULL */
  float head_weight;           /* dpm_head_weight */
  int head_part;               /* 5 (1 for 12 parts, 11 for 22 parts) in the reference */
  const float *head;           /* [H][W] head DPM scores, or NULL */
  float unary_weight;          /* dpm_unary_weight */
  int unary_rot;               /* do_dpm_rot */
  const float *unary;          /* [n_parts][unary_rot ? R : 1][H][W], or NULL */
  const int *is_detect;        /* [n_parts] PartDef::is_detect flags (host), or NULL: all */
} pa_dpm_terms;

pa_status pa_add_dpm_scores(pa_ctx *ctx, const pa_exp_param *ep, const pa_dpm_terms *dt,
                            int n_parts, int root, float *log_unary, int H, int W, int mem);

/* ------------------------------------------- hypothesis suppression */

/* nms_recursive (libPictStruct/objectdetect_aux.cpp:407-451), as
 * saveRecoResults (:453-600) runs it on the merged root hypotheses of an
 * image: hypotheses sorted by descending score; suppressed[j] = 1 when an
 * earlier hypothesis i has (x_i - x_j)^2 / e1 + (y_i - y_j)^2 / e2 < 1 with
 * e1 = (0.5 * scale_i * train_object_width)^2, e2 likewise with the height
 * (the differences in float, the rest in double, as the reference types it).
 * Scores out of descending order are PA_ERR_INVALID (the reference asserts).
 * `mem` tells where the five arrays lie; n = 0 is a no-op.  The pair test is
 * O(n^2) double divisions, so n is capped at PA_NMS_MAX_HYPS (the reference
 * runs it on one image's root hypotheses, a few hundred); larger n is
 * PA_ERR_INVALID. */
#define PA_NMS_MAX_HYPS 65536
pa_status pa_nms_recursive(pa_ctx *ctx, int n, const float *x, const float *y, const float *scale,
                           const float *score, double train_object_width,
                           double train_object_height, int *suppressed, int mem);

/* nms_recursive of libNms, rectangle form (libNms/nms.cpp:132-225): n
 * rectangles as corners rects[n][4][2] (x, y; double), sorted by descending
 * score; suppressed[j] = 1 when an earlier rectangle i has
 * dx^2 / e1 + dy^2 / e2 < ellipse_size^2, with e1 = |r1 - r0|^2,
 * e2 = |r1 - r2|^2 of rectangle i, (dx, dy) the offset of j's centre from
 * i's (centres: the mean of the four corners) projected on i's unit edges
 * (r1 - r0) / sqrt(e1) and (r1 - r2) / sqrt(e2), every step in double.  The
 * hypothesis-list form (:58-84) is pa_rect_from_hyp per hypothesis, then
 * this call; the reference's default ellipse_size is 0.5 (:45-56).  Scores
 * out of descending order are PA_ERR_INVALID; n <= PA_NMS_MAX_HYPS; `mem`
 * tells where rects, score and suppressed lie. */
pa_status pa_nms_rects(pa_ctx *ctx, int n, const double *rects, const double *score,
                       double ellipse_size, int *suppressed, int mem);

/* rect_from_hyp (libNms/nms.cpp:23-56): the upright rectangle of a
 * hypothesis (x, y, scale as stored, float), height (int)(scale *
 * reference_height) and width (int)(scale * reference_width) pixels,
 * corners rect[4][2] = centre -+ half width, -+ half height in the
 * reference's order.  Host memory; no context. */
void pa_rect_from_hyp(float x, float y, float scale, double reference_height,
                      double reference_width, double *rect);

/* ---------------------------------------------------- learned unary */

/* No counterpart in the reference: a convolutional network that maps a
 * descriptor field to the log scores of the part detectors and can stand in
 * for the AdaBoost unaries (computeScoreGrid + clip_scores_fill + log) of
 * chosen parts.  Layers, all with zero padding and bias:
 *   1x1 conv  dim -> 64, ReLU
 *   3x3 conv  64 -> 64, ReLU   (three layers)
 *   3x3 conv  64 -> n_parts     (log scores)
 * BF16 weights and activations, FP32 accumulation on the tensor cores,
 * FP32 master weights trained with Adam.  Parameters, flat FP32, in order:
 *   W0 [64][dim], b0 [64], then for l = 1..3: Wl [64][9][64], bl [64],
 *   then W4 [n_parts][9][64], b4 [n_parts]
 * (weights [out channel][tap (dy, dx row-major)][in channel]).
 * Fields are NHWC: [n_fields][ny][nx][dim], dim a multiple of 64, FP32 or
 * BF16, 16-byte aligned.  All data pointers of these calls are device
 * pointers. */
typedef struct pa_unary_net pa_unary_net;

typedef struct {
  float lr, beta1, beta2, eps;
} pa_adam_param;

/* Weights drawn from `seed` (He-normal; the output layer's scaled by 0.1),
 * zero biases; Adam state zero. */
pa_status pa_unary_net_create(pa_ctx *ctx, int dim, int n_parts, uint64_t seed,
                              pa_unary_net **out);
pa_status pa_unary_net_destroy(pa_ctx *ctx, pa_unary_net *net);
/* Number of parameters; copies them to host `params` when not NULL. */
pa_status pa_unary_net_get_params(pa_ctx *ctx, const pa_unary_net *net, float *params,
                                  int64_t *n_params);
/* Replaces the parameters (host array) and resets the Adam state. */
pa_status pa_unary_net_set_params(pa_ctx *ctx, pa_unary_net *net, const float *params);
/* Log scores (exp_out = 0) or scores (exp_out = 1) of the n_parts outputs:
 * element (field f, part p, row y, column x) at
 * out[f * out_field_stride + p * out_part_stride + y * nx + x]. */
pa_status pa_unary_net_forward(pa_ctx *ctx, pa_unary_net *net, const void *fields, int fields_bf16,
                               int n_fields, int ny, int nx, float *out, int64_t out_field_stride,
                               int64_t out_part_stride, int exp_out);
/* Mean squared error against the log of AdaBoost score grids, and its
 * gradient with respect to every parameter (kept in the net; copied to host
 * `grads` when not NULL).  scores: [n_parts][n_fields][ny][nx] as
 * pa_score_grids writes them (normalised); the target of a cell is
 * log(s) for s > 0, log(1e-4) for s < 0 (clip_scores_fill), and cells with
 * s == 0 (LOG_ZERO) are left out.  loss = sum of squared errors over
 * (n_fields * n_parts * ny * nx). */
pa_status pa_unary_net_backward(pa_ctx *ctx, pa_unary_net *net, const void *fields,
                                int fields_bf16, const float *scores, int n_fields, int ny,
                                int nx, double *loss, float *grads);
/* One Adam step with the gradient of the last pa_unary_net_backward. */
pa_status pa_unary_net_adam(pa_ctx *ctx, pa_unary_net *net, const pa_adam_param *opt);

/* The image loop of findObjectDataset (objectdetect_aux.cpp:322-406) over
 * images of uneven sizes and rotation counts, as pa_find_obj_multi, with the
 * message passing of all images of a wave in ONE persistent launch:
 * no counterpart in the reference, which loops over images serially.
 * Per wave (up to images_per_wave images, bounded by device memory) the
 * unaries run as one launch per group of images that share sizes; then a
 * persistent kernel drains a device work queue of tiles -- the rows and
 * column bands of every message of every image and the root combinations --
 * in the order of computeRootPosteriorRot (objectdetect_findrot.cpp:582-658
 * upward, then computePartMarginals :192-236 downward), each image's tree
 * order enforced by per-job completion counters in device memory; then the
 * root posterior, log-partition and local maxima per group.  Every device
 * wait is bounded by wait_timeout_ms: a wait that runs out abandons the
 * wave and the call returns PA_ERR_TIMEOUT.  Row-tile widths are chosen per
 * shape class by measuring candidates once (autotune) and cached in the
 * context.  Results equal pa_find_obj_multi's bit for bit.  Device inputs
 * only; images whose messages need the full-covariance or tensor-core
 * paths are processed as pa_find_obj_multi does. */
typedef struct {
  int images_per_wave;    /* images per persistent launch (0: 32) */
  double wait_timeout_ms; /* bound of each dependency wait (<= 0: 20000 ms) */
  int autotune;           /* measure row-tile widths per shape class (1) or take the default (0) */
  int hold_start;         /* diagnostic: the host never opens the queue's start gate, so every
                           * wait runs out (tests of the time-out path); 0 normally */
} pa_queue_opts;
void pa_queue_opts_default(pa_queue_opts *o);
pa_status pa_find_obj_queue(pa_ctx *ctx, int n_images, const pa_image *imgs,
                            const pa_classifier *const *cls, int n_cls, const pa_queue_opts *opts);

/* pa_find_obj_batch with the net as the unary of the parts whose
 * part_on_net[p] is non-zero (all parts when part_on_net is NULL) and the
 * AdaBoost classifiers cls[p] for the others.
 *   fields  [n_images][R][ny][nx][dim] BF16, read by the net (may be NULL
 *           when no part is on the net)
 *   desc    the same descriptors in FP32 for the AdaBoost parts (may be
 *           NULL when every part is on the net)
 * Device pointers (mem = PA_MEM_DEVICE) only. */
pa_status pa_find_obj_batch_learned(pa_ctx *ctx, const pa_exp_param *ep, int n_images,
                                    const pa_tree *trees, int flip, pa_unary_net *net,
                                    const int *part_on_net, const pa_classifier *const *cls,
                                    int n_cls, const void *fields, const float *desc, int ny,
                                    int nx, int dim, const double *Tig, int tig_shared, int H,
                                    int W, const pa_ps_outputs *out);

#ifdef __cplusplus
}
#endif
#endif /* PARTAPP_GB300_H_ */
