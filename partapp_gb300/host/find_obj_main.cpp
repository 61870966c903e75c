// find_obj_main.cpp -- `partapp_find_obj --find_obj`: the --find_obj mode of
// the reference's partapp binary (apps/partapp/main.cpp, findObjectDataset)
// over an experiment directory of plain files:
//
//   exp.txt        "key value" lines: num_rotation_steps, min_part_rotation,
//                  max_part_rotation, object_scale, strip_border_detections,
//                  roi_save_num_samples, use_pairwise, interpolate, height,
//                  width, grid_ny, grid_nx, dim, n_classifiers, n_images
//   tig.txt        9 numbers: grid -> image transform, row-major 3x3
//   joints.txt     "n_parts root", then n_parts is_upright flags, then one
//                  line per joint: child parent ocx ocy opx opy C00 C01 C10
//                  C11 rot_mean rot_sigma (radians; joints_<i>.txt if present
//                  overrides it for image i)
//   class_<c>.txt  AdaBoost classifier c in the reference's text format
//                  (libAdaBoost/AdaBoost.cc:295-338)
//   desc_<i>.bin   float32 [R][grid_ny][grid_nx][dim] descriptors of image i
//
// With --from_images the descriptors are computed on the GPU from grey
// images (partdetect, the force_recompute_scores branch of findObjectDataset):
//   img_<i>.pgm    8-bit binary PGM (P5) grey image i
//   windows.txt    one line per classifier: window_size_x window_size_y
//                  pos_offset_x pos_offset_y (PartWindowParam)
//   exp.txt        additionally desc_step, desc_size, window_desc_step_ratio
//                  (AbcDetectorParam) and, for several scales, num_scale_steps,
//                  min_object_scale, max_object_scale (in place of
//                  object_scale); height, width, grid_*, dim and tig.txt are
//                  not used
//   --detection_masks_dir DIR   DIR/detection_mask_imgidx<NNNNN>.mat per image
//                  (exp_param.detection_masks_dir, partdetect_test.cpp:89-99)
//
// With --scoregrid_dir DIR the unaries come from the score grids the
// reference's part detector saved (the default branch of findObjectDataset,
// force_recompute_scores off: findObjectImageRotJoints with bLoadScoreGrid):
//   DIR/imgidx<i>-pidx<p>-o<flip>-scoregrid.mat   cell_scoregrid, transform_Ti2,
//                                                 transform_T2g (compressed or not)
//   exp.txt, joints.txt as above; the image size is exp.txt's height and width,
//   or the header of img_<i>.pgm when that file exists; classifiers, tig.txt and
//   descriptors are not used.
//
// The poselet-conditioned extra unary terms (findObjectImageRotJoints,
// objectdetect_findrot.cpp:855-948) are added, in the --scoregrid_dir and
// --from_images modes, when asked for:
//   --pred_dir DIR --pred_rot_weight w   rotation score (testlist_params_rot_imgidx_<i>.mat)
//   --pred_dir DIR --pred_pos_weight w --torso_det_dir DIR [--rootidx_det k]
//                                        position score around the torso detection
//   --torso_prior FILE --torso_prior_weight w   torso position prior
// and, before them, the DPM score terms (objectdetect_findrot.cpp:883-914):
//   --dpm_torso_dir DIR [--dpm_torso_weight w]  torso grid on the root part
//   --dpm_unary_dir DIR --use_dpm_head [--dpm_head_weight w]   head grid
//   --dpm_unary_dir DIR --use_dpm_unary [--dpm_unary_weight w] [--dpm_rot]
//                                        per-part grids (per rotation)
//
// The joints come from joints.txt (above), or from the reference's own
// experiment files: --part_conf FILE (PartConfig, protobuf text format) with
// --spatial_dir DIR (joint_<child>_<parent>.mat, load_joint) and, for
// mixtures of pairwise terms (num_joint_types > 1), --pred_dir DIR
// (testlist_pred_pwise_imgidx_<i>.mat, clusidx_test -> joint_<c>_<p>_tidx_<t>.mat).
// --joints_dump prints the joints as loaded (no GPU needed).
// --mask_dump S H W (with --detection_masks_dir DIR --first i) prints image i's
// detection masks as loaded for S scales of H x W (no GPU needed).
//
// --mat_dump FILE prints every variable of a MAT-file (name, class, dims and
// values in MATLAB's column-major order, cells one by one).
//
// Writes, into --outdir, the reference's result files pose_est_imgidx<NNNN>.mat
// (best_conf) and, with --save_marginals, log_part_posterior_final_*.mat, plus
// best_conf_<i>.txt (one PartHyp::toVect line per part), log_z_<i>.txt and
// part_hyps_<i>.txt.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "mat_io.hpp"
#include "partapp_gpu.hpp"

using namespace partapp_gpu;

namespace {

std::string read_file(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

bool exists(const std::string &path) { return std::ifstream(path).good(); }

std::map<std::string, double> read_kv(const std::string &path) {
  std::map<std::string, double> kv;
  std::istringstream in(read_file(path));
  std::string k;
  double v;
  while (in >> k >> v) kv[k] = v;
  return kv;
}

double need(const std::map<std::string, double> &kv, const std::string &k) {
  auto it = kv.find(k);
  if (it == kv.end()) throw std::runtime_error("exp.txt: missing " + k);
  return it->second;
}

void read_joints(const std::string &path, PartConfig &pc, std::vector<Joint> &js) {
  std::istringstream in(read_file(path));
  int P = 0;
  in >> P >> pc.rootpart_idx;
  if (!in || P < 1) throw std::runtime_error(path + ": bad header");
  pc.is_upright.assign(P, 0);
  for (int p = 0; p < P; ++p) in >> pc.is_upright[p];
  js.clear();
  for (int j = 0; j < P - 1; ++j) {
    Joint J;
    in >> J.child_idx >> J.parent_idx >> J.offset_c[0] >> J.offset_c[1] >> J.offset_p[0] >>
        J.offset_p[1] >> J.C[0] >> J.C[1] >> J.C[2] >> J.C[3] >> J.rot_mean >> J.rot_sigma;
    if (!in) throw std::runtime_error(path + ": bad joint line");
    js.push_back(J);
  }
}

// Where the joints come from: the reference's experiment files (the part
// configuration in protobuf text format and joint_<c>_<p>[_tidx_<t>].mat
// under the spatial directory, mixture components from predictFactors'
// output under --pred_dir) when --part_conf is given, else joints.txt and
// the per-image joints_<i>.txt.
struct JointSource {
  std::string part_conf, spatial_dir, pred_dir;
  PartConfigFile pcf;

  void load_base(const std::string &expdir, PartConfig &pc, std::vector<Joint> &js) {
    if (part_conf.empty()) {
      read_joints(expdir + "/joints.txt", pc, js);
      return;
    }
    if (spatial_dir.empty()) throw std::runtime_error("--part_conf needs --spatial_dir");
    pcf = parsePartConfig(read_file(part_conf));
    pc = partConfigOf(pcf);
    js = loadJoints(pcf, spatial_dir);
  }
  std::vector<Joint> for_image(const std::string &expdir, int img,
                               const std::vector<Joint> &base) const {
    if (!part_conf.empty()) {
      if (pred_dir.empty() || pcf.joints.empty() || pcf.joints[0].num_joint_types <= 1) return base;
      return loadJoints(pcf, spatial_dir, loadJointTypes(pcf, pred_dir, img));
    }
    const std::string jp = expdir + "/joints_" + std::to_string(img) + ".txt";
    if (!exists(jp)) return base;
    PartConfig pc;
    std::vector<Joint> js;
    read_joints(jp, pc, js);
    return js;
  }
};

void dump_joints(const PartConfig &pc, const std::vector<Joint> &js) {
  std::printf("parts %d root %d upright", pc.part_size(), pc.rootpart_idx);
  for (int u : pc.is_upright) std::printf(" %d", u);
  std::printf("\n");
  for (const Joint &J : js)
    std::printf("joint %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
                J.child_idx, J.parent_idx, J.offset_c[0], J.offset_c[1], J.offset_p[0],
                J.offset_p[1], J.C[0], J.C[1], J.C[2], J.C[3], J.rot_mean, J.rot_sigma);
}

// Binary 8-bit PGM (P5) -> grey levels 0..255 as float (the reference loads
// images as float grey levels, kma::load_convert_gray_image).
std::vector<float> read_pgm(const std::string &path, int &h, int &w) {
  const std::string d = read_file(path);
  size_t pos = 0;
  auto token = [&]() -> std::string {
    for (;;) {
      while (pos < d.size() && std::isspace((unsigned char)d[pos])) ++pos;
      if (pos < d.size() && d[pos] == '#') {
        while (pos < d.size() && d[pos] != '\n') ++pos;
        continue;
      }
      break;
    }
    const size_t b = pos;
    while (pos < d.size() && !std::isspace((unsigned char)d[pos])) ++pos;
    return d.substr(b, pos - b);
  };
  if (token() != "P5") throw std::runtime_error(path + ": not a binary PGM (P5)");
  w = std::atoi(token().c_str());
  h = std::atoi(token().c_str());
  const int maxval = std::atoi(token().c_str());
  ++pos;  // the single whitespace after maxval
  if (w < 1 || h < 1 || maxval < 1 || maxval > 255 || d.size() < pos + (size_t)w * h)
    throw std::runtime_error(path + ": unsupported or truncated PGM");
  std::vector<float> img((size_t)w * h);
  for (size_t k = 0; k < img.size(); ++k) img[k] = (float)(unsigned char)d[pos + k];
  return img;
}

void write_outputs(const std::string &outdir, int img, bool flip, const FindObjResult &r) {
  const std::string tag = std::to_string(img);
  std::ofstream bc(outdir + "/best_conf_" + tag + ".txt");
  bc.precision(9);
  for (const PartHyp &h : r.best_conf) {
    const auto v = h.toVect();
    for (size_t k = 0; k < v.size(); ++k) bc << (k ? " " : "") << v[k];
    bc << "\n";
  }
  std::ofstream lz(outdir + "/log_z_" + tag + ".txt");
  lz.precision(17);
  for (double z : r.log_z) lz << z << "\n";
  if (!saveResults(outdir, img, flip, r))
    throw std::runtime_error("cannot write the .mat results to " + outdir);
  std::ofstream ph(outdir + "/part_hyps_" + tag + ".txt");
  ph.precision(9);
  for (size_t p = 0; p < r.part_hyps.size(); ++p)
    for (const PartHyp &h : r.part_hyps[p])
      ph << p << " " << h.m_rotidx << " " << h.m_x << " " << h.m_y << " " << h.m_score << "\n";
}

bool pgm_size(const std::string &path, int &h, int &w) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::string magic;
  in >> magic;
  auto next_int = [&](int &v) {
    in >> std::ws;
    while (in.peek() == '#') {
      std::string line;
      std::getline(in, line);
      in >> std::ws;
    }
    in >> v;
  };
  int maxv = 0;
  next_int(w);
  next_int(h);
  next_int(maxv);
  return magic == "P5" && (bool)in && w > 0 && h > 0;
}

void dump_array(const MatArray &a, const std::string &indent) {
  std::cout << indent << "var " << (a.name.empty() ? "-" : a.name) << " class " << a.mx_class
            << " dims";
  for (size_t d : a.dims) std::cout << ' ' << d;
  std::cout << '\n';
  if (a.is_cell()) {
    for (const MatArray &c : a.cells) dump_array(c, indent + "  ");
    return;
  }
  std::cout << indent;
  char buf[32];
  for (double v : a.re) {
    std::snprintf(buf, sizeof buf, "%.17g ", v);
    std::cout << buf;
  }
  std::cout << '\n';
}

void usage() {
  std::cout << "usage: partapp_find_obj --find_obj --expdir DIR [--outdir DIR] [--first i]\n"
               "                        [--numimgs n] [--batch b] [--flip] [--device d]\n"
               "                        [--save_marginals] [--from_images [--detection_masks_dir DIR]\n"
               "                         | --scoregrid_dir DIR]\n"
               "                        [--pred_dir DIR --pred_rot_weight w --pred_pos_weight w\n"
               "                         --torso_det_dir DIR --rootidx_det k]\n"
               "                        [--torso_prior FILE --torso_prior_weight w]\n"
               "                        [--dpm_torso_dir DIR --dpm_torso_weight w]\n"
               "                        [--dpm_unary_dir DIR --use_dpm_head --dpm_head_weight w\n"
               "                         --use_dpm_unary --dpm_unary_weight w --dpm_rot]\n"
               "                        [--part_conf FILE --spatial_dir DIR [--pred_dir DIR]]\n"
               "       partapp_find_obj --mask_dump S H W --detection_masks_dir DIR [--first i]\n"
               "       partapp_find_obj --joints_dump [--expdir DIR | --part_conf FILE\n"
               "                        --spatial_dir DIR [--pred_dir DIR]] [--first i --numimgs n]\n"
               "       partapp_find_obj --mat_dump FILE\n";
}

}  // namespace

int main(int argc, char **argv) {
  std::string expdir, outdir, scoregrid_dir, pred_dir, torso_det_dir, torso_prior, masks_dir;
  float rot_w = 0.f, pos_w = 0.f, torso_w = 0.f;
  int rootidx_det = -1;
  DpmOptions dpm;
  int first = 0, numimgs = -1, batch = 1, device = 0;
  bool find_obj = false, flip = false, save_marg = false, from_images = false, joints_dump = false;
  bool mask_dump = false;
  int mask_dims[3] = {0, 0, 0};
  JointSource jsrc;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw std::runtime_error("missing value after " + a);
      return argv[++i];
    };
    if (a == "--find_obj") find_obj = true;
    else if (a == "--expdir") expdir = next();
    else if (a == "--outdir") outdir = next();
    else if (a == "--first") first = std::atoi(next().c_str());
    else if (a == "--numimgs") numimgs = std::atoi(next().c_str());
    else if (a == "--batch") batch = std::atoi(next().c_str());
    else if (a == "--device") device = std::atoi(next().c_str());
    else if (a == "--flip") flip = true;
    else if (a == "--save_marginals") save_marg = true;
    else if (a == "--from_images") from_images = true;
    else if (a == "--scoregrid_dir") scoregrid_dir = next();
    else if (a == "--detection_masks_dir") masks_dir = next();
    else if (a == "--part_conf") jsrc.part_conf = next();
    else if (a == "--spatial_dir") jsrc.spatial_dir = next();
    else if (a == "--joints_dump") joints_dump = true;
    else if (a == "--mask_dump") {
      mask_dims[0] = std::atoi(next().c_str());
      mask_dims[1] = std::atoi(next().c_str());
      mask_dims[2] = std::atoi(next().c_str());
      mask_dump = true;
    }
    else if (a == "--pred_dir") jsrc.pred_dir = pred_dir = next();
    else if (a == "--pred_rot_weight") rot_w = (float)std::atof(next().c_str());
    else if (a == "--pred_pos_weight") pos_w = (float)std::atof(next().c_str());
    else if (a == "--torso_det_dir") torso_det_dir = next();
    else if (a == "--rootidx_det") rootidx_det = std::atoi(next().c_str());
    else if (a == "--torso_prior") torso_prior = next();
    else if (a == "--torso_prior_weight") torso_w = (float)std::atof(next().c_str());
    else if (a == "--dpm_torso_dir") dpm.torso_dir = next();
    else if (a == "--dpm_torso_weight") dpm.torso_weight = (float)std::atof(next().c_str());
    else if (a == "--dpm_unary_dir") dpm.unary_dir = next();
    else if (a == "--use_dpm_head") dpm.head = true;
    else if (a == "--dpm_head_weight") dpm.head_weight = (float)std::atof(next().c_str());
    else if (a == "--use_dpm_unary") dpm.unary = true;
    else if (a == "--dpm_unary_weight") dpm.unary_weight = (float)std::atof(next().c_str());
    else if (a == "--dpm_rot") dpm.rot = true;
    else if (a == "--mat_dump") {
      try {
        for (const MatArray &v : mat_read(next())) dump_array(v, "");
      } catch (const std::exception &ex) {
        std::cerr << "partapp_find_obj: " << ex.what() << "\n";
        return 1;
      }
      return 0;
    }
    else if (a == "--help" || a == "-h") { usage(); return 0; }
    else { std::cerr << "unknown option " << a << "\n"; usage(); return 2; }
  }
  if (mask_dump) {
    try {
      const int S = mask_dims[0], H = mask_dims[1], W = mask_dims[2];
      if (S < 1 || H < 1 || W < 1 || masks_dir.empty())
        throw std::runtime_error("--mask_dump needs S H W >= 1 and --detection_masks_dir");
      const std::vector<float> m = loadDetectionMask(masks_dir, first, S, H, W);
      for (int sc = 0; sc < S; ++sc) {
        std::printf("scale %d\n", sc);
        for (int y = 0; y < H; ++y) {
          for (int x = 0; x < W; ++x)
            std::printf(x ? " %.9g" : "%.9g", (double)m[((size_t)sc * H + y) * W + x]);
          std::printf("\n");
        }
      }
    } catch (const std::exception &ex) {
      std::cerr << "partapp_find_obj: " << ex.what() << "\n";
      return 1;
    }
    return 0;
  }
  if (joints_dump) {
    try {
      PartApp app;
      jsrc.load_base(expdir, app.m_part_conf, app.m_joints);
      dump_joints(app.m_part_conf, app.m_joints);
      for (int i = first; i < first + std::max(0, numimgs); ++i) {
        std::printf("image %d\n", i);
        dump_joints(app.m_part_conf, jsrc.for_image(expdir, i, app.m_joints));
      }
    } catch (const std::exception &ex) {
      std::cerr << "partapp_find_obj: " << ex.what() << "\n";
      return 1;
    }
    return 0;
  }
  if (!find_obj || expdir.empty()) {
    usage();
    return find_obj ? 2 : 0;
  }
  if (outdir.empty()) outdir = expdir;
  try {
    const auto kv = read_kv(expdir + "/exp.txt");
    PartApp app;
    ExpParam &e = app.m_exp_param;
    e.num_rotation_steps = (int)need(kv, "num_rotation_steps");
    e.min_part_rotation = (float)need(kv, "min_part_rotation");
    e.max_part_rotation = (float)need(kv, "max_part_rotation");
    if (!(from_images && kv.count("num_scale_steps")))
      e.min_object_scale = e.max_object_scale = (float)need(kv, "object_scale");
    e.strip_border_detections = (float)need(kv, "strip_border_detections");
    e.roi_save_num_samples = (int)need(kv, "roi_save_num_samples");
    e.use_pairwise = need(kv, "use_pairwise") != 0;
    e.interpolate = need(kv, "interpolate") != 0;
    // the saved-score-grid branch needs no classifiers
    const int n_cls = scoregrid_dir.empty() ? (int)need(kv, "n_classifiers") : 0;
    const int n_images = (int)need(kv, "n_images");
    if (numimgs < 0) numimgs = n_images - first;
    if (first < 0 || first + numimgs > n_images || batch < 1)
      throw std::runtime_error("image range outside the experiment");
    if (from_images) {
      app.m_abc_param.desc_step = (int)need(kv, "desc_step");
      app.m_abc_param.desc_size = (int)need(kv, "desc_size");
      app.m_abc_param.window_desc_step_ratio = need(kv, "window_desc_step_ratio");
      if (kv.count("num_scale_steps")) {  // several scales (partdetect_test.cpp:116)
        e.num_scale_steps = (int)need(kv, "num_scale_steps");
        e.min_object_scale = (float)need(kv, "min_object_scale");
        e.max_object_scale = (float)need(kv, "max_object_scale");
      }
      std::istringstream win(read_file(expdir + "/windows.txt"));
      for (int c = 0; c < n_cls; ++c) {
        PartWindow pw;
        win >> pw.window_size_x >> pw.window_size_y >> pw.pos_offset_x >> pw.pos_offset_y;
        if (!win) throw std::runtime_error("windows.txt: need one line per classifier");
        app.m_window_param.push_back(pw);
      }
      jsrc.load_base(expdir, app.m_part_conf, app.m_joints);
      Context ctx(device);
      std::vector<std::unique_ptr<AdaBoostClassifier>> abc;
      for (int c = 0; c < n_cls; ++c) {
        abc.emplace_back(new AdaBoostClassifier(ctx, read_file(expdir + "/class_" + std::to_string(c) + ".txt")));
        app.m_abc.push_back(abc.back().get());
      }
      for (int i = first; i < first + numimgs; ++i) {
        int h = 0, w = 0;
        const std::vector<float> img = read_pgm(expdir + "/img_" + std::to_string(i) + ".pgm", h, w);
        const std::vector<Joint> joints = jsrc.for_image(expdir, i, app.m_joints);
        ExtraUnaryParams extra = loadExtraUnaryParams(
            i, app.m_part_conf.part_size(), app.m_part_conf.rootpart_idx, pred_dir, rot_w, pos_w,
            torso_det_dir, rootidx_det, torso_prior, torso_w);
        loadDpmScores(extra, i, app.m_part_conf.part_size(), app.m_exp_param.c().num_rotation_steps,
                      h, w, dpm);
        app.m_extra = &extra;
        std::vector<float> mask;
        if (!masks_dir.empty())
          mask = loadDetectionMask(masks_dir, i, std::max(1, app.m_exp_param.num_scale_steps), h,
                                   w);
        app.m_detection_mask = masks_dir.empty() ? nullptr : &mask;
        const FindObjResult r = findObjectImageFromImage(ctx, app, flip, joints, img.data(), h, w,
                                                         save_marg);
        write_outputs(outdir, i, flip, r);
        std::cout << "find_obj: image " << i << " (" << w << "x" << h << ") done\n";
      }
      return 0;
    }
    if (!scoregrid_dir.empty()) {
      jsrc.load_base(expdir, app.m_part_conf, app.m_joints);
      const int P = app.m_part_conf.part_size();
      Context ctx(device);
      for (int i = first; i < first + numimgs; ++i) {
        int h = 0, w = 0;
        if (!pgm_size(expdir + "/img_" + std::to_string(i) + ".pgm", h, w)) {
          h = (int)need(kv, "height");
          w = (int)need(kv, "width");
        }
        const std::vector<Joint> joints = jsrc.for_image(expdir, i, app.m_joints);
        std::vector<ScoreGridSet> parts;
        for (int p = 0; p < P; ++p)
          parts.push_back(loadScoreGrid(scoreGridFileName(scoregrid_dir, i, p, flip)));
        ExtraUnaryParams extra =
            loadExtraUnaryParams(i, P, app.m_part_conf.rootpart_idx, pred_dir, rot_w, pos_w,
                                 torso_det_dir, rootidx_det, torso_prior, torso_w);
        loadDpmScores(extra, i, P, app.m_exp_param.c().num_rotation_steps, h, w, dpm);
        app.m_extra = &extra;
        const FindObjResult r =
            findObjectImageFromScoreGrids(ctx, app, flip, joints, parts, h, w, save_marg);
        write_outputs(outdir, i, flip, r);
        std::cout << "find_obj: image " << i << " (" << w << "x" << h << ", saved score grids) done\n";
      }
      return 0;
    }
    const int H = (int)need(kv, "height"), W = (int)need(kv, "width");
    const int ny = (int)need(kv, "grid_ny"), nx = (int)need(kv, "grid_nx");
    const int dim = (int)need(kv, "dim");
    const int R = e.num_rotation_steps;

    double Tig[9];
    {
      std::istringstream in(read_file(expdir + "/tig.txt"));
      for (double &t : Tig) in >> t;
      if (!in) throw std::runtime_error("tig.txt: need 9 numbers");
    }
    jsrc.load_base(expdir, app.m_part_conf, app.m_joints);

    Context ctx(device);
    std::vector<std::unique_ptr<AdaBoostClassifier>> abc;
    for (int c = 0; c < n_cls; ++c) {
      abc.emplace_back(new AdaBoostClassifier(ctx, read_file(expdir + "/class_" + std::to_string(c) + ".txt")));
      app.m_abc.push_back(abc.back().get());
    }

    const size_t per_img = (size_t)R * ny * nx * dim;
    for (int i0 = first; i0 < first + numimgs; i0 += batch) {
      const int nb = std::min(batch, first + numimgs - i0);
      std::vector<float> desc(per_img * nb);
      std::vector<std::vector<Joint>> joints;
      for (int b = 0; b < nb; ++b) {
        const int img = i0 + b;
        const std::string d = read_file(expdir + "/desc_" + std::to_string(img) + ".bin");
        if (d.size() != per_img * sizeof(float))
          throw std::runtime_error("desc_" + std::to_string(img) + ".bin: wrong size");
        std::memcpy(desc.data() + per_img * b, d.data(), d.size());
        joints.push_back(jsrc.for_image(expdir, img, app.m_joints));
      }
      const auto res =
          findObjectDataset(ctx, app, flip, joints, desc.data(), nb, ny, nx, dim, Tig, H, W, save_marg);
      for (int b = 0; b < nb; ++b) write_outputs(outdir, i0 + b, flip, res[b]);
      std::cout << "find_obj: images " << i0 << ".." << i0 + nb - 1 << " done\n";
    }
  } catch (const std::exception &ex) {
    std::cerr << "partapp_find_obj: " << ex.what() << "\n";
    return 1;
  }
  return 0;
}
