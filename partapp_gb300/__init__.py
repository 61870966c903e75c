"""partapp_gb300 -- GB300 implementation of partapp's --find_obj hot path.

Python binding of the C-ABI in include/partapp_gb300.h (libpartapp_gb300.so,
built by partapp_gb300.build).  The names mirror the reference's C++ entry
points:

  Context.score_grids          computeScoreGrid + evaluateFeaturePoint
                               (libPartDetect/partdetect_test.cpp:344-405,
                                libAdaBoost/AdaBoost.h:131-160)
  Context.score_grids_window   the FeatureGrid::concatenate form
  Context.unary_maps           grid -> image + clip_scores_fill + computeLogGrid
  Context.rot_joint_marginal   computeRotJointMarginal
                               (libPictStruct/objectdetect_findrot.cpp:292-456)
  Context.compute_root_posterior_rot
                               computeRootPosteriorRot + computePartMarginals
                               (objectdetect_findrot.cpp:124-286, 470-727)
  Context.find_obj             findObjectImageRotJoints with fresh scores
  Context.find_obj_batch       many images per call
  UnaryNet                     the learned unary (no reference counterpart):
                               forward, backward, Adam, and
                               Context.find_obj_batch_learned

Arrays: numpy arrays are host memory (copied through the device workspace);
torch CUDA tensors are used in place as device memory.  There is no CPU
fallback: without the built library or a GPU every compute call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpartapp_gb300.so")

PA_OK, PA_ERR_INVALID, PA_ERR_UNSUPPORTED, PA_ERR_CUDA, PA_ERR_NOMEM, PA_ERR_NUMERIC, \
    PA_ERR_TIMEOUT = range(7)
PA_MEM_DEVICE, PA_MEM_HOST = 0, 1
LOG_ZERO = -1e6
NO_CLASS_VALUE = 0.0
NOALLOC_MAX_CELLS = 2097152  # PA_NOALLOC_MAX_CELLS

# every symbol include/partapp_gb300.h declares
EXPORTS = (
    "pa_ctx_create", "pa_ctx_destroy", "pa_ctx_set_stream", "pa_ctx_synchronize",
    "pa_last_error", "pa_status_string", "pa_ctx_kernel_launches", "pa_ctx_enable_timing",
    "pa_ctx_timing_reset", "pa_ctx_timing_count", "pa_ctx_timing_get", "pa_exp_param_default",
    "pa_classifier_create", "pa_classifier_parse", "pa_classifier_destroy",
    "pa_classifier_info", "pa_score_grids", "pa_score_grids_window", "pa_unary_maps",
    "pa_ps_infer", "pa_rot_joint_marginal", "pa_rot_joint_marginal_noalloc", "pa_find_obj",
    "pa_feature_grid_size", "pa_descriptor_grid", "pa_partdetect",
    "pa_find_obj_batch", "pa_gemm_bf16", "pa_ctx_set_message_math", "pa_find_obj_multi",
    "pa_unary_net_create", "pa_unary_net_destroy", "pa_unary_net_get_params",
    "pa_unary_net_set_params", "pa_unary_net_forward", "pa_unary_net_backward",
    "pa_unary_net_adam", "pa_find_obj_batch_learned", "pa_add_extra_unaries", "pa_add_dpm_scores",
    "pa_nms_recursive", "pa_queue_opts_default", "pa_find_obj_queue", "pa_nms_rects",
    "pa_rect_from_hyp", "pa_descriptor_grid_masked", "pa_partdetect_masked",
    "pa_find_obj_scales",
)
PA_MSG_FP32, PA_MSG_BF16_TENSOR = 0, 1


class QueueOpts(C.Structure):
    """pa_queue_opts."""
    _fields_ = [("images_per_wave", C.c_int), ("wait_timeout_ms", C.c_double),
                ("autotune", C.c_int), ("hold_start", C.c_int)]


class Image(C.Structure):
    _fields_ = [("ep", C.c_void_p), ("tree", C.c_void_p), ("flip", C.c_int), ("desc", C.c_void_p),
                ("ny", C.c_int), ("nx", C.c_int), ("dim", C.c_int), ("Tig", C.c_void_p),
                ("tig_shared", C.c_int), ("H", C.c_int), ("W", C.c_int), ("out", C.c_void_p)]


class ScaleFields(C.Structure):
    """pa_scale_fields."""
    _fields_ = [("desc", C.c_void_p), ("ny", C.c_int), ("nx", C.c_int), ("dim", C.c_int),
                ("Tig", C.c_void_p), ("tig_shared", C.c_int)]


class PaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class ExpParam(C.Structure):
    _fields_ = [("num_rotation_steps", C.c_int), ("min_part_rotation", C.c_float),
                ("max_part_rotation", C.c_float), ("min_object_scale", C.c_float),
                ("max_object_scale", C.c_float), ("strip_border_detections", C.c_float),
                ("roi_save_num_samples", C.c_int), ("use_pairwise", C.c_int),
                ("interpolate", C.c_int), ("num_scale_steps", C.c_int)]


class AbcParam(C.Structure):
    _fields_ = [("desc_step", C.c_int), ("desc_size", C.c_int),
                ("window_desc_step_ratio", C.c_double)]


class PartWindow(C.Structure):
    _fields_ = [("window_size_x", C.c_int), ("window_size_y", C.c_int),
                ("pos_offset_x", C.c_double), ("pos_offset_y", C.c_double)]


class Stump(C.Structure):
    _fields_ = [("f", C.c_int32), ("p", C.c_float), ("theta", C.c_float), ("alpha", C.c_float)]


class Tree(C.Structure):
    _fields_ = [("n_parts", C.c_int), ("root", C.c_int), ("is_upright", C.POINTER(C.c_int)),
                ("n_joints", C.c_int), ("child", C.POINTER(C.c_int)),
                ("parent", C.POINTER(C.c_int)), ("offset_c", C.POINTER(C.c_double)),
                ("offset_p", C.POINTER(C.c_double)), ("C", C.POINTER(C.c_double)),
                ("rot_mean", C.POINTER(C.c_double)), ("rot_sigma", C.POINTER(C.c_double))]


class PartHyp(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("scaleidx", "scale", "rotidx", "rot", "x", "y", "score")]


class AdamParam(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float)]


class ExtraUnary(C.Structure):
    _fields_ = [("rot_weight", C.c_float), ("rot_params", C.c_void_p), ("pos_weight", C.c_float),
                ("pos_params", C.c_void_p), ("root_det_x", C.c_double), ("root_det_y", C.c_double),
                ("torso_weight", C.c_float), ("torso_prior", C.c_void_p),
                ("is_detect", C.c_void_p)]


class DpmTerms(C.Structure):
    _fields_ = [("torso_weight", C.c_float), ("torso", C.c_void_p), ("head_weight", C.c_float),
                ("head_part", C.c_int), ("head", C.c_void_p), ("unary_weight", C.c_float),
                ("unary_rot", C.c_int), ("unary", C.c_void_p), ("is_detect", C.c_void_p)]


class PsOutputs(C.Structure):
    _fields_ = [("log_marg", C.c_void_p), ("root_post", C.c_void_p),
                ("best", C.POINTER(PartHyp)), ("part_hyps", C.POINTER(PartHyp)),
                ("n_part_hyps", C.POINTER(C.c_int)), ("root_hyps", C.POINTER(C.c_float)),
                ("n_root_hyps", C.POINTER(C.c_int)), ("log_z", C.POINTER(C.c_double)),
                ("msg_max", C.POINTER(C.c_double))]


_lib = None


def load_library():
    """Load libpartapp_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"partapp_gb300: native library missing at {LIB_PATH}; "
                          "build it with `python -m partapp_gb300.build`")
    L = C.CDLL(LIB_PATH)
    vp, ip, dp, fp = C.c_void_p, C.c_int, C.c_double, C.c_float
    P = C.POINTER
    L.pa_ctx_create.argtypes = [ip, P(vp)]
    L.pa_ctx_destroy.argtypes = [vp]
    L.pa_ctx_set_stream.argtypes = [vp, vp]
    L.pa_ctx_synchronize.argtypes = [vp]
    L.pa_last_error.argtypes = [vp]
    L.pa_last_error.restype = C.c_char_p
    L.pa_status_string.argtypes = [ip]
    L.pa_status_string.restype = C.c_char_p
    L.pa_ctx_kernel_launches.argtypes = [vp]
    L.pa_ctx_kernel_launches.restype = C.c_uint64
    L.pa_ctx_enable_timing.argtypes = [vp, ip]
    L.pa_ctx_timing_reset.argtypes = [vp]
    L.pa_ctx_timing_count.argtypes = [vp]
    L.pa_ctx_timing_get.argtypes = [vp, ip, P(C.c_char_p), P(dp), P(C.c_uint64)]
    L.pa_exp_param_default.argtypes = [P(ExpParam)]
    L.pa_exp_param_default.restype = None
    L.pa_classifier_create.argtypes = [vp, ip, P(Stump), ip, P(vp)]
    L.pa_classifier_parse.argtypes = [vp, C.c_char_p, C.c_size_t, P(vp)]
    L.pa_classifier_destroy.argtypes = [vp, vp]
    L.pa_classifier_info.argtypes = [vp, P(ip), P(ip), P(fp)]
    L.pa_score_grids.argtypes = [vp, P(vp), ip, vp, ip, ip, ip, ip, ip, vp, ip]
    L.pa_score_grids_window.argtypes = [vp, P(vp), ip, vp, vp, ip, ip, ip, ip, ip, ip, dp, ip,
                                        vp, ip]
    L.pa_unary_maps.argtypes = [vp, vp, ip, ip, ip, ip, P(dp), ip, ip, ip, ip, vp, ip]
    L.pa_ps_infer.argtypes = [vp, P(ExpParam), P(Tree), ip, ip, vp, ip, ip, P(PsOutputs), ip]
    L.pa_feature_grid_size.argtypes = [ip, ip, P(dp), P(dp), dp, P(ip), P(ip)]
    L.pa_descriptor_grid.argtypes = [vp, vp, ip, ip, P(dp), P(dp), dp, ip, vp, vp, ip]
    L.pa_partdetect.argtypes = [vp, P(ExpParam), vp, ip, ip, ip, vp, ip, P(PartWindow),
                                P(AbcParam), vp, ip]
    L.pa_descriptor_grid_masked.argtypes = [vp, vp, ip, ip, P(dp), P(dp), dp, ip, vp, P(ip), vp,
                                            vp, ip]
    L.pa_partdetect_masked.argtypes = [vp, P(ExpParam), vp, ip, ip, ip, vp, ip, P(PartWindow),
                                       P(AbcParam), vp, vp, ip]
    L.pa_rot_joint_marginal.argtypes = [vp, P(ExpParam), vp, vp, ip, ip, ip, P(dp), P(dp), P(dp),
                                        dp, dp, dp, ip, ip]
    L.pa_gemm_bf16.argtypes = [vp, vp, C.c_int64, vp, C.c_int64, vp, C.c_int64, ip, ip, ip, ip]
    L.pa_ctx_set_message_math.argtypes = [vp, ip]
    L.pa_find_obj_multi.argtypes = [vp, ip, P(Image), P(vp), ip, ip]
    L.pa_find_obj_queue.argtypes = [vp, ip, P(Image), P(vp), ip, P(QueueOpts)]
    L.pa_queue_opts_default.argtypes = [P(QueueOpts)]
    L.pa_queue_opts_default.restype = None
    L.pa_rot_joint_marginal_noalloc.argtypes = [P(ExpParam), vp, vp, ip, ip, ip, P(dp), P(dp),
                                                 P(dp), dp, dp, dp, vp]
    L.pa_find_obj.argtypes = [vp, P(ExpParam), P(Tree), ip, P(vp), ip, vp, ip, ip, ip, P(dp), ip,
                              ip, ip, vp, P(PsOutputs), ip]
    L.pa_find_obj_batch.argtypes = [vp, P(ExpParam), ip, P(Tree), ip, P(vp), ip, vp, ip, ip, ip,
                                    P(dp), ip, ip, ip, vp, P(PsOutputs), ip]
    L.pa_find_obj_scales.argtypes = [vp, P(ExpParam), P(Tree), ip, P(vp), ip, P(ScaleFields), ip,
                                     ip, P(PsOutputs), ip]
    L.pa_add_extra_unaries.argtypes = [vp, P(ExpParam), P(ExtraUnary), ip, ip, vp, ip, ip, ip]
    L.pa_add_dpm_scores.argtypes = [vp, P(ExpParam), P(DpmTerms), ip, ip, vp, ip, ip, ip]
    L.pa_nms_recursive.argtypes = [vp, ip, vp, vp, vp, vp, dp, dp, vp, ip]
    L.pa_nms_rects.argtypes = [vp, ip, vp, vp, dp, vp, ip]
    L.pa_rect_from_hyp.argtypes = [C.c_float, C.c_float, C.c_float, dp, dp, vp]
    L.pa_rect_from_hyp.restype = None
    L.pa_unary_net_create.argtypes = [vp, ip, ip, C.c_uint64, P(vp)]
    L.pa_unary_net_destroy.argtypes = [vp, vp]
    L.pa_unary_net_get_params.argtypes = [vp, vp, vp, P(C.c_int64)]
    L.pa_unary_net_set_params.argtypes = [vp, vp, vp]
    L.pa_unary_net_forward.argtypes = [vp, vp, vp, ip, ip, ip, ip, vp, C.c_int64, C.c_int64, ip]
    L.pa_unary_net_backward.argtypes = [vp, vp, vp, ip, vp, ip, ip, ip, P(dp), vp]
    L.pa_unary_net_adam.argtypes = [vp, vp, P(AdamParam)]
    L.pa_find_obj_batch_learned.argtypes = [vp, P(ExpParam), ip, P(Tree), ip, vp, vp, P(vp), ip,
                                            vp, vp, ip, ip, ip, P(dp), ip, ip, ip, P(PsOutputs)]
    for name in EXPORTS:
        getattr(L, name)  # every declared entry point must resolve
    _lib = L
    return L


def exp_param(R=24, min_rot=-180.0, max_rot=180.0, scale=1.0, strip=0.0, local_max=1000,
              use_pairwise=True, interpolate=True, n_scales=1, scale_range=None) -> ExpParam:
    """n_scales > 1 needs scale_range = (min_object_scale, max_object_scale)."""
    lo, hi = (scale, scale) if scale_range is None else scale_range
    return ExpParam(int(R), float(min_rot), float(max_rot), float(lo), float(hi),
                    float(strip), int(local_max), int(bool(use_pairwise)), int(bool(interpolate)),
                    int(n_scales))


def rect_from_hyp(x, y, scale, reference_height, reference_width) -> np.ndarray:
    """libNms rect_from_hyp: the corners [4][2] (double) of the upright
    rectangle of a hypothesis (x, y, scale as stored, float)."""
    out = np.zeros(8, np.float64)
    load_library().pa_rect_from_hyp(float(x), float(y), float(scale), float(reference_height),
                                    float(reference_width), out.ctypes.data)
    return out.reshape(4, 2)


def _is_torch(a):
    return type(a).__module__.startswith("torch")


class _Buf:
    """Holds a numpy or torch buffer and its pointer + memory space."""

    def __init__(self, a, dtype):
        if _is_torch(a):
            import torch

            tdt = {np.float32: torch.float32, np.float64: torch.float64, np.uint8: torch.uint8}[dtype]
            if not a.is_cuda:
                raise ValueError("torch tensors must live on the GPU")
            if a.dtype != tdt or not a.is_contiguous():
                raise ValueError(f"expected a contiguous {tdt} CUDA tensor")
            self.arr, self.ptr, self.mem = a, a.data_ptr(), PA_MEM_DEVICE
        else:
            arr = np.ascontiguousarray(a, dtype=dtype)
            self.arr, self.ptr, self.mem = arr, arr.ctypes.data, PA_MEM_HOST


def _mask_buf(mask, like: _Buf, shape):
    """A float32 detection mask in the memory space of `like`, checked for shape."""
    if mask is None:
        return None
    if like.mem == PA_MEM_DEVICE and not _is_torch(mask):
        import torch

        mask = torch.as_tensor(np.ascontiguousarray(mask, dtype=np.float32), device=like.arr.device)
    elif like.mem == PA_MEM_HOST and _is_torch(mask):
        mask = mask.detach().cpu().numpy()
    if _is_torch(mask):
        import torch

        mask = mask.to(torch.float32).contiguous()
    m = _Buf(mask, np.float32)
    if tuple(m.arr.shape) != tuple(shape):
        raise ValueError(f"detection mask must be {tuple(shape)}, got {tuple(m.arr.shape)}")
    return m


def _empty_like_space(shape, mem, like=None):
    if mem == PA_MEM_DEVICE:
        import torch

        return torch.empty(shape, dtype=torch.float32, device=like.device)
    return np.empty(shape, dtype=np.float32)


class _TreeHolder:
    def __init__(self, tree):
        self.is_upright = np.ascontiguousarray(tree["is_upright"], dtype=np.int32)
        self.child = np.ascontiguousarray(tree["child"], dtype=np.int32)
        self.parent = np.ascontiguousarray(tree["parent"], dtype=np.int32)
        self.offset_c = np.ascontiguousarray(tree["offset_c"], dtype=np.float64).reshape(-1)
        self.offset_p = np.ascontiguousarray(tree["offset_p"], dtype=np.float64).reshape(-1)
        self.C = np.ascontiguousarray(tree["C"], dtype=np.float64).reshape(-1)
        self.rot_mean = np.ascontiguousarray(tree["rot_mean"], dtype=np.float64)
        self.rot_sigma = np.ascontiguousarray(tree["rot_sigma"], dtype=np.float64)
        pi = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self.s = Tree(int(tree["n_parts"]), int(tree["root"]), pi(self.is_upright),
                      len(self.child), pi(self.child), pi(self.parent), pd(self.offset_c),
                      pd(self.offset_p), pd(self.C), pd(self.rot_mean), pd(self.rot_sigma))


class Classifier:
    """An AdaBoost classifier resident on the device (pa_classifier)."""

    def __init__(self, ctx: "Context", handle, keep=None):
        self.ctx, self.h, self._keep = ctx, handle, keep

    @classmethod
    def from_stumps(cls, ctx, f, p, theta, alpha, dim):
        n = len(f)
        arr = (Stump * n)()
        for i in range(n):
            arr[i] = Stump(int(f[i]), float(p[i]), float(theta[i]), float(alpha[i]))
        h = C.c_void_p()
        ctx._check(ctx.L.pa_classifier_create(ctx.h, int(dim), arr, n, C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def parse(cls, ctx, text: str):
        b = text.encode()
        h = C.c_void_p()
        ctx._check(ctx.L.pa_classifier_parse(ctx.h, b, len(b), C.byref(h)))
        return cls(ctx, h)

    def info(self):
        d, n, s = C.c_int(), C.c_int(), C.c_float()
        self.ctx.L.pa_classifier_info(self.h, C.byref(d), C.byref(n), C.byref(s))
        return d.value, n.value, s.value

    def close(self):
        if self.h:
            self.ctx.L.pa_classifier_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A pa_ctx: one device, one stream, its own workspace.

    The context issues its work on torch's current stream of `device` (when
    torch with CUDA is present), so CUDA tensors produced by torch just before
    a call are complete when the call reads them, and torch sees the outputs
    in order; set_stream() moves it to another stream.  Without torch the
    context keeps its own stream."""

    def __init__(self, device: int = 0):
        self.L = load_library()
        h = C.c_void_p()
        st = self.L.pa_ctx_create(int(device), C.byref(h))
        if st != PA_OK:
            raise PaError(st, "pa_ctx_create failed (no CUDA device?)")
        self.h = h
        try:
            import torch

            if torch.cuda.is_available():
                self.set_stream(torch.cuda.current_stream(int(device)).cuda_stream)
        except ImportError:
            pass

    def close(self):
        if getattr(self, "h", None):
            self.L.pa_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != PA_OK:
            raise PaError(st, self.L.pa_last_error(self.h).decode())

    def set_stream(self, stream_ptr: int):
        self._check(self.L.pa_ctx_set_stream(self.h, C.c_void_p(stream_ptr)))

    def synchronize(self):
        self._check(self.L.pa_ctx_synchronize(self.h))

    @property
    def kernel_launches(self) -> int:
        return int(self.L.pa_ctx_kernel_launches(self.h))

    def enable_timing(self, on: bool = True):
        self._check(self.L.pa_ctx_enable_timing(self.h, int(on)))

    def reset_timing(self):
        self._check(self.L.pa_ctx_timing_reset(self.h))

    def kernel_times(self) -> dict:
        """{kernel: (total_ms, launches)} accumulated while timing was on."""
        out = {}
        for i in range(self.L.pa_ctx_timing_count(self.h)):
            nm, ms, n = C.c_char_p(), C.c_double(), C.c_uint64()
            self._check(self.L.pa_ctx_timing_get(self.h, i, C.byref(nm), C.byref(ms), C.byref(n)))
            out[nm.value.decode()] = (ms.value, int(n.value))
        return out

    # ---------------------------------------------------------- unaries
    def classifiers(self, models) -> list:
        """Upload {f, p, theta, alpha} arrays of shape [n_parts][n_stumps]."""
        D = int(models.get("D", int(np.max(models["f"])) + 1))
        return [Classifier.from_stumps(self, models["f"][i], models["p"][i], models["theta"][i],
                                       models["alpha"][i], D) for i in range(len(models["f"]))]

    @staticmethod
    def _cls_array(cls_list):
        return (C.c_void_p * len(cls_list))(*[c.h for c in cls_list])

    def score_grids(self, cls_list, desc, normalize=True):
        """desc [n_fields][ny][nx][dim] -> scores [n_parts][n_fields][ny][nx]."""
        d = _Buf(desc, np.float32)
        nf, ny, nx, dim = d.arr.shape
        out = _empty_like_space((len(cls_list), nf, ny, nx), d.mem, d.arr)
        o = _Buf(out, np.float32)
        self._check(self.L.pa_score_grids(self.h, self._cls_array(cls_list), len(cls_list), d.ptr,
                                          nf, ny, nx, dim, int(normalize), o.ptr, d.mem))
        return out

    def score_grids_window(self, cls_list, cells, valid, gx, gy, grid_step, normalize=True):
        c = _Buf(cells, np.float32)
        v = _Buf(valid, np.uint8)
        nf, ny, nx, dc = c.arr.shape
        out = _empty_like_space((len(cls_list), nf, ny, nx), c.mem, c.arr)
        o = _Buf(out, np.float32)
        self._check(self.L.pa_score_grids_window(self.h, self._cls_array(cls_list),
                                                 len(cls_list), c.ptr, v.ptr, nf, ny, nx, dc,
                                                 int(gx), int(gy), float(grid_step),
                                                 int(normalize), o.ptr, c.mem))
        return out

    def unary_maps(self, scores, Tig, H, W, interpolate=True):
        """scores [P][R][ny][nx] -> log unaries [P][R][H][W]."""
        s = _Buf(scores, np.float32)
        P, R, ny, nx = s.arr.shape
        T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(-1)
        shared = int(T.size == 9)
        out = _empty_like_space((P, R, H, W), s.mem, s.arr)
        o = _Buf(out, np.float32)
        self._check(self.L.pa_unary_maps(self.h, s.ptr, P, R, ny, nx,
                                         T.ctypes.data_as(C.POINTER(C.c_double)), shared,
                                         int(interpolate), H, W, o.ptr, s.mem))
        return out

    # ------------------------------------------------------ descriptors
    def descriptor_grid(self, image, x_axis, y_axis, desc_step, desc_size, mask=None, roi=None):
        """computeDescriptorGrid with SHAPEv5 on a grey image [h][w] (numpy or
        CUDA tensor): returns (cells [ny][nx][96] f32, valid [ny][nx] u8) in
        the image's memory space.  mask: detection mask [h][w] (0: no
        descriptor there) or None; roi: (x, y, width, height) as QRect(x, y,
        width, height), or None for the default QRect(0, 0, w - 1, h - 1)."""
        im = _Buf(image, np.float32)
        h, w = im.arr.shape
        ax = np.ascontiguousarray(x_axis, dtype=np.float64).reshape(2)
        ay = np.ascontiguousarray(y_axis, dtype=np.float64).reshape(2)
        pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        nx, ny = C.c_int(), C.c_int()
        self._check(self.L.pa_feature_grid_size(w, h, pd(ax), pd(ay), float(desc_step),
                                                C.byref(nx), C.byref(ny)))
        cells = _empty_like_space((ny.value, nx.value, 96), im.mem, im.arr)
        if im.mem == PA_MEM_DEVICE:
            import torch
            valid = torch.empty((ny.value, nx.value), dtype=torch.uint8, device=im.arr.device)
            vptr = valid.data_ptr()
        else:
            valid = np.empty((ny.value, nx.value), np.uint8)
            vptr = valid.ctypes.data
        mk = _mask_buf(mask, im, (h, w))
        rr = None if roi is None else (C.c_int * 4)(*[int(v) for v in roi])
        self._check(self.L.pa_descriptor_grid_masked(
            self.h, im.ptr, h, w, pd(ax), pd(ay), float(desc_step), int(desc_size),
            None if mk is None else mk.ptr, rr, _Buf(cells, np.float32).ptr, vptr, im.mem))
        return cells, valid

    def partdetect(self, exp: ExpParam, image, cls_list, windows, desc_step, desc_size,
                   ratio=1.0, flip=False, mask=None):
        """partdetect_dense + clip/log on one grey image [h][w] (numpy or CUDA
        tensor): windows = [(window_size_x, window_size_y, pos_offset_x,
        pos_offset_y)] per classifier; mask: detection masks [S][h][w] (one
        per scale) or None; returns log unaries [n][R][h][w], or
        [n][S][R][h][w] for num_scale_steps = S > 1."""
        im = _Buf(image, np.float32)
        h, w = im.arr.shape
        n = len(cls_list)
        R = exp.num_rotation_steps
        S = max(1, exp.num_scale_steps)
        wins = (PartWindow * n)(*[PartWindow(int(a[0]), int(a[1]), float(a[2]), float(a[3]))
                                  for a in windows])
        abc = AbcParam(int(desc_step), int(desc_size), float(ratio))
        out = _empty_like_space((n, S, R, h, w) if S > 1 else (n, R, h, w), im.mem, im.arr)
        mk = _mask_buf(mask, im, (S, h, w))
        self._check(self.L.pa_partdetect_masked(
            self.h, C.byref(exp), im.ptr, h, w, int(bool(flip)), self._cls_array(cls_list), n,
            wins, C.byref(abc), None if mk is None else mk.ptr, _Buf(out, np.float32).ptr,
            im.mem))
        return out

    # ---------------------------------------------------------- messages
    def rot_joint_marginal(self, exp: ExpParam, child, offset_c, offset_p, Cmat, rot_mean,
                           rot_sigma, scale=1.0, is_sparse=False):
        """computeRotJointMarginal; is_sparse = bIsSparse (TM_DIRECT forward
        rotation of a full covariance)."""
        c = _Buf(child, np.float32)
        R, H, W = c.arr.shape
        out = _empty_like_space((R, H, W), c.mem, c.arr)
        o = _Buf(out, np.float32)
        dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        oc, op, Cm = dp(offset_c), dp(offset_p), dp(Cmat)
        pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._check(self.L.pa_rot_joint_marginal(self.h, C.byref(exp), c.ptr, o.ptr, R, H, W,
                                                 pd(oc), pd(op), pd(Cm), float(rot_mean),
                                                 float(rot_sigma), float(scale),
                                                 int(is_sparse), c.mem))
        return out

    def _outputs(self, P, R, H, W, K, mem, like, want_marg=True, want_root=True, S=0):
        """S = 0: one-scale shapes; S >= 1: [P][S][R][H][W] / [S][H][W] maps."""
        n = max(S, 1)
        res = dict(best=(PartHyp * P)(), log_z=np.zeros(n * P),
                   msg_max=np.zeros(n * max(1, 2 * (P - 1))),
                   n_part_hyps=np.zeros(P, dtype=np.int32), n_root_hyps=np.zeros(1, np.int32),
                   part_hyps=(PartHyp * max(1, P * K))(), root_hyps=np.zeros((1000, 4), np.float32))
        mshape = (P, S, R, H, W) if S else (P, R, H, W)
        rshape = (S, H, W) if S else (H, W)
        res["log_marg"] = _empty_like_space(mshape, mem, like) if want_marg else None
        res["root_post"] = _empty_like_space(rshape, mem, like) if want_root else None
        ptr = lambda a: None if a is None else _Buf(a, np.float32).ptr
        o = PsOutputs(ptr(res["log_marg"]), ptr(res["root_post"]), res["best"], res["part_hyps"],
                      res["n_part_hyps"].ctypes.data_as(C.POINTER(C.c_int)),
                      res["root_hyps"].ctypes.data_as(C.POINTER(C.c_float)),
                      res["n_root_hyps"].ctypes.data_as(C.POINTER(C.c_int)),
                      res["log_z"].ctypes.data_as(C.POINTER(C.c_double)),
                      res["msg_max"].ctypes.data_as(C.POINTER(C.c_double)))
        return res, o

    @staticmethod
    def _finish(res, P):
        res["best_conf"] = np.array([[h.scaleidx, h.scale, h.rotidx, h.rot, h.x, h.y, h.score]
                                     for h in res.pop("best")], dtype=np.float32)
        ph = np.frombuffer(res["part_hyps"], dtype=np.float32)
        res["part_hyps"] = ph.reshape(P, -1, 7).copy() if ph.size >= 7 * P else ph.reshape(0, 7)
        res["root_hyps"] = res["root_hyps"][: int(res["n_root_hyps"][0])]
        return res

    def _image_list(self, images, want_marg):
        keep, imgs, results = [], [], []
        mem = None
        for im in images:
            d = _Buf(im["desc"], np.float32)
            mem = d.mem if mem is None else mem
            if d.mem != mem:
                raise ValueError("all descriptors must live in the same memory space")
            R, ny, nx, dim = d.arr.shape
            th = _TreeHolder(im["tree"])
            P = th.s.n_parts
            T = np.ascontiguousarray(im["Tig"], dtype=np.float64).reshape(-1)
            exp = im["exp"]
            res, o = self._outputs(P, R, im["H"], im["W"], exp.roi_save_num_samples, d.mem, d.arr,
                                   want_marg)
            keep += [d, th, T, exp, o]
            imgs.append(Image(C.addressof(exp), C.addressof(th.s), int(im.get("flip", False)),
                              d.ptr, ny, nx, dim, T.ctypes.data, 1, im["H"], im["W"],
                              C.addressof(o)))
            results.append((res, P))
        return (Image * len(imgs))(*imgs), results, mem, keep

    def find_obj_multi(self, images, cls_list, want_marg=False):
        """images: list of dicts {exp, tree, desc [R][ny][nx][dim], Tig, H, W,
        flip=False} of possibly different sizes and rotation counts; all
        descriptors numpy (host) or all CUDA tensors (device)."""
        arr, results, mem, keep = self._image_list(images, want_marg)
        self._check(self.L.pa_find_obj_multi(self.h, len(arr), arr, self._cls_array(cls_list),
                                             len(cls_list), mem))
        return [self._finish(res, P) for res, P in results]

    def find_obj_queue(self, images, cls_list, want_marg=False, images_per_wave=32,
                       wait_timeout_ms=20000.0, autotune=True, hold_start=False):
        """pa_find_obj_queue: as find_obj_multi (CUDA tensors only), the
        message passing of each wave of images in one persistent launch."""
        arr, results, mem, keep = self._image_list(images, want_marg)
        if mem != PA_MEM_DEVICE:
            raise ValueError("find_obj_queue takes CUDA tensors")
        o = QueueOpts(int(images_per_wave), float(wait_timeout_ms), int(bool(autotune)),
                      int(bool(hold_start)))
        self._check(self.L.pa_find_obj_queue(self.h, len(arr), arr, self._cls_array(cls_list),
                                             len(cls_list), C.byref(o)))
        return [self._finish(res, P) for res, P in results]

    def set_message_math(self, mode):
        """PA_MSG_FP32 (default) or PA_MSG_BF16_TENSOR for the spatial filter
        of diagonal-covariance messages."""
        self._check(self.L.pa_ctx_set_message_math(self.h, int(mode)))

    def gemm_bf16(self, A, B, out=None):
        """C = A @ B.T on the tensor cores: A [M][K], B [N][K] bf16 CUDA
        tensors (K contiguous, K padded to a multiple of 8 by the caller);
        returns C [M][N] fp32 (or fills `out`)."""
        import torch

        assert A.is_cuda and B.is_cuda and A.dtype == torch.bfloat16 and B.dtype == torch.bfloat16
        M, K = A.shape
        N = B.shape[0]
        C_ = out if out is not None else torch.empty((M, N), dtype=torch.float32, device=A.device)
        self._check(self.L.pa_gemm_bf16(self.h, A.data_ptr(), A.stride(0), B.data_ptr(),
                                        B.stride(0), C_.data_ptr(), C_.stride(0), M, N, K, -1))
        return C_

    def gemm_bf16_banded(self, A, B, band):
        """C = A @ B.T for a banded A (A[m][k] = 0 for |k - m| > band)."""
        import torch

        M, K = A.shape
        N = B.shape[0]
        C_ = torch.empty((M, N), dtype=torch.float32, device=A.device)
        self._check(self.L.pa_gemm_bf16(self.h, A.data_ptr(), A.stride(0), B.data_ptr(),
                                        B.stride(0), C_.data_ptr(), C_.stride(0), M, N, K,
                                        int(band)))
        return C_

    def add_extra_unaries(self, exp: ExpParam, log_unary, root, rot=None, pos=None, torso=None,
                          is_detect=None):
        """findObjectImageRotJoints' poselet-conditioned terms, in place on
        log_unary [P][S][R][H][W] or [P][R][H][W] (numpy or CUDA tensor).
        rot = (weight, params [P][2]: mean (rad), variance); pos = (weight,
        params [P][4]: mu_x, mu_y, var_x, var_y, (det_x, det_y)); torso =
        (weight, params [4])."""
        u = _Buf(log_unary, np.float32)
        shp = u.arr.shape
        P, H, W = shp[0], shp[-2], shp[-1]
        keep = []

        def arr(a, dt=np.float64):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data

        ex = ExtraUnary()
        if rot is not None:
            ex.rot_weight, ex.rot_params = float(rot[0]), arr(rot[1])
        if pos is not None:
            ex.pos_weight, ex.pos_params = float(pos[0]), arr(pos[1])
            ex.root_det_x, ex.root_det_y = float(pos[2][0]), float(pos[2][1])
        if torso is not None:
            ex.torso_weight, ex.torso_prior = float(torso[0]), arr(torso[1])
        if is_detect is not None:
            ex.is_detect = arr(is_detect, np.int32)
        self._check(self.L.pa_add_extra_unaries(self.h, C.byref(exp), C.byref(ex), P, int(root),
                                                u.ptr, H, W, u.mem))
        if u.mem == PA_MEM_HOST and u.arr is not log_unary:
            np.copyto(log_unary, u.arr)
        return log_unary

    def add_dpm_scores(self, exp: ExpParam, log_unary, root, torso=None, head=None, unary=None,
                       is_detect=None):
        """findObjectImageRotJoints' DPM terms, in place on log_unary
        [P][S][R][H][W] or [P][R][H][W] (numpy or CUDA tensor; the grids are
        taken to the same place).  torso = (weight, grid [H][W]); head =
        (weight, part, grid [H][W]); unary = (weight, grids [P][R or 1][H][W]);
        grids hold raw DPM scores."""
        u = _Buf(log_unary, np.float32)
        shp = u.arr.shape
        P, R, H, W = shp[0], shp[-3], shp[-2], shp[-1]
        keep = []

        def grid(a):
            if u.mem == PA_MEM_DEVICE:
                import torch

                t = torch.as_tensor(a, dtype=torch.float32, device=log_unary.device).contiguous()
                keep.append(t)
                return t.data_ptr()
            a = np.ascontiguousarray(a, dtype=np.float32)
            keep.append(a)
            return a.ctypes.data

        dt = DpmTerms()
        for name, term, idx in (("torso", torso, 1), ("head", head, 2)):
            if term is not None and tuple(term[idx].shape) != (H, W):
                raise ValueError(f"the {name} DPM grid must be [H][W] = [{H}][{W}]")
        if torso is not None:
            dt.torso_weight, dt.torso = float(torso[0]), grid(torso[1])
        if head is not None:
            dt.head_weight, dt.head_part, dt.head = float(head[0]), int(head[1]), grid(head[2])
        if unary is not None:
            g = unary[1]
            if tuple(g.shape) not in ((P, R, H, W), (P, 1, H, W)):
                raise ValueError("unary DPM grids must be [P][R or 1][H][W]")
            dt.unary_weight, dt.unary_rot, dt.unary = float(unary[0]), int(g.shape[1] == R and R > 1), grid(g)
        if is_detect is not None:
            isd = np.ascontiguousarray(is_detect, dtype=np.int32)
            keep.append(isd)
            dt.is_detect = isd.ctypes.data
        self._check(self.L.pa_add_dpm_scores(self.h, C.byref(exp), C.byref(dt), P, int(root),
                                             u.ptr, H, W, u.mem))
        if u.mem == PA_MEM_HOST and u.arr is not log_unary:
            np.copyto(log_unary, u.arr)
        return log_unary

    def nms_recursive(self, x, y, scale, score, train_object_width, train_object_height):
        """nms_recursive over hypotheses sorted by descending score (numpy
        arrays or CUDA tensors, all alike): suppressed flags, bool [n] (int32
        CUDA tensor for tensor input)."""
        bufs = [_Buf(v, np.float32) for v in (x, y, scale, score)]
        n = int(bufs[0].arr.shape[0])
        if any(int(b.arr.shape[0]) != n or b.mem != bufs[0].mem for b in bufs):
            raise ValueError("x, y, scale and score must have one length and one place")
        if bufs[0].mem == PA_MEM_DEVICE:
            import torch

            out = torch.zeros(n, dtype=torch.int32, device=x.device)
            ptr = out.data_ptr()
        else:
            out = np.zeros(n, np.int32)
            ptr = out.ctypes.data
        self._check(self.L.pa_nms_recursive(self.h, n, *[b.ptr for b in bufs],
                                            float(train_object_width), float(train_object_height),
                                            ptr, bufs[0].mem))
        return out if bufs[0].mem == PA_MEM_DEVICE else out.astype(bool)

    def nms_rects(self, rects, scores, ellipse_size=0.5):
        """libNms nms_recursive on rectangles [n][4][2] (double corners) sorted
        by descending score (numpy arrays or CUDA tensors, alike): suppressed
        flags, bool [n] (int32 CUDA tensor for tensor input)."""
        r = _Buf(rects, np.float64)
        sc = _Buf(scores, np.float64)
        n = int(sc.arr.shape[0])
        if tuple(r.arr.shape) != (n, 4, 2) or r.mem != sc.mem:
            raise ValueError("rects [n][4][2] and scores [n] must be alike")
        if sc.mem == PA_MEM_DEVICE:
            import torch

            out = torch.zeros(n, dtype=torch.int32, device=scores.device)
            ptr = out.data_ptr()
        else:
            out = np.zeros(n, np.int32)
            ptr = out.ctypes.data
        self._check(self.L.pa_nms_rects(self.h, n, r.ptr, sc.ptr, float(ellipse_size), ptr, sc.mem))
        return out if sc.mem == PA_MEM_DEVICE else out.astype(bool)

    def compute_root_posterior_rot(self, exp: ExpParam, tree, log_unary, flip=False,
                                   want_marg=True, is_sparse=False):
        """log_unary [P][R][H][W] or, for num_scale_steps = S, [P][S][R][H][W]
        (after clip_scores_fill + computeLogGrid); is_sparse = bIsSparse of
        the upward messages.  With the 5-d form the maps come back as
        [P][S][R][H][W] / [S][H][W] and log_z as [S][P]."""
        u = _Buf(log_unary, np.float32)
        multi = len(u.arr.shape) == 5
        P, S, R, H, W = u.arr.shape if multi else (u.arr.shape[0], 1) + tuple(u.arr.shape[1:])
        if S != max(1, exp.num_scale_steps):
            raise ValueError("log_unary has a different number of scales than exp")
        th = _TreeHolder(tree)
        res, o = self._outputs(P, R, H, W, exp.roi_save_num_samples, u.mem, u.arr, want_marg,
                               S=S if multi else 0)
        self._check(self.L.pa_ps_infer(self.h, C.byref(exp), C.byref(th.s), int(flip),
                                       int(is_sparse), u.ptr, H, W, C.byref(o), u.mem))
        if multi:
            res["log_z"] = res["log_z"].reshape(S, P)
            res["msg_max"] = res["msg_max"].reshape(S, -1)
        return self._finish(res, P)

    def find_obj(self, exp: ExpParam, tree, cls_list, desc, Tig, H, W, flip=False,
                 want_marg=True):
        """desc [R][ny][nx][dim] -> marginals, argmax, root posterior of one image."""
        d = _Buf(desc, np.float32)
        R, ny, nx, dim = d.arr.shape
        th = _TreeHolder(tree)
        P = th.s.n_parts
        T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(-1)
        res, o = self._outputs(P, R, H, W, exp.roi_save_num_samples, d.mem, d.arr, want_marg)
        self._check(self.L.pa_find_obj(self.h, C.byref(exp), C.byref(th.s), int(flip),
                                       self._cls_array(cls_list), len(cls_list), d.ptr, ny, nx,
                                       dim, T.ctypes.data_as(C.POINTER(C.c_double)),
                                       int(T.size == 9), H, W, None, C.byref(o), d.mem))
        return self._finish(res, P)

    def find_obj_scales(self, exp: ExpParam, tree, cls_list, descs, Tigs, H, W, flip=False,
                        want_marg=True):
        """descs: one [R][ny][nx][dim] array per scale (grid sizes may differ),
        Tigs: one grid -> image transform per scale ([9] or [P][R][9]); the
        maps come back as [P][S][R][H][W] / [S][H][W], log_z as [S][P]."""
        S = max(1, exp.num_scale_steps)
        if len(descs) != S or len(Tigs) != S:
            raise ValueError("one descriptor array and one Tig per scale")
        bufs = [_Buf(d, np.float32) for d in descs]
        if len({b.mem for b in bufs}) != 1:
            raise ValueError("all scales' descriptors in one memory space")
        th = _TreeHolder(tree)
        P = th.s.n_parts
        R = bufs[0].arr.shape[0]
        Ts = [np.ascontiguousarray(T, dtype=np.float64).reshape(-1) for T in Tigs]
        fields = (ScaleFields * S)(*[
            ScaleFields(b.ptr, b.arr.shape[1], b.arr.shape[2], b.arr.shape[3], T.ctypes.data,
                        int(T.size == 9)) for b, T in zip(bufs, Ts)])
        res, o = self._outputs(P, R, H, W, exp.roi_save_num_samples, bufs[0].mem, bufs[0].arr,
                               want_marg, S=S if S > 1 else 0)
        self._check(self.L.pa_find_obj_scales(self.h, C.byref(exp), C.byref(th.s), int(flip),
                                              self._cls_array(cls_list), len(cls_list), fields,
                                              H, W, C.byref(o), bufs[0].mem))
        if S > 1:
            res["log_z"] = res["log_z"].reshape(S, P)
            res["msg_max"] = res["msg_max"].reshape(S, -1)
        return self._finish(res, P)

    def find_obj_batch(self, exp: ExpParam, trees, cls_list, desc, Tig, H, W, flip=False,
                       want_marg=False, want_root=False, scores_out=None):
        """desc [B][R][ny][nx][dim]; trees: list of B tree dicts (same topology).
        cls_list may hold more classifiers than the tree has parts; the first
        n_parts feed the tree, all are evaluated (scores_out, if given, is
        [n_cls][B*R][ny][nx] in the same memory space as desc)."""
        d = _Buf(desc, np.float32)
        B, R, ny, nx, dim = d.arr.shape
        ths = [_TreeHolder(t) for t in trees]
        arr = (Tree * B)(*[t.s for t in ths])
        P = ths[0].s.n_parts
        T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(-1)
        results, outs = [], (PsOutputs * B)()
        for i in range(B):
            res, o = self._outputs(P, R, H, W, exp.roi_save_num_samples, d.mem, d.arr, want_marg,
                                   want_root)
            results.append(res)
            outs[i] = o
        so = None if scores_out is None else _Buf(scores_out, np.float32).ptr
        self._check(self.L.pa_find_obj_batch(self.h, C.byref(exp), B, arr, int(flip),
                                             self._cls_array(cls_list), len(cls_list), d.ptr, ny,
                                             nx, dim, T.ctypes.data_as(C.POINTER(C.c_double)),
                                             int(T.size == 9), H, W, so, outs, d.mem))
        return [self._finish(r, P) for r in results]


def _dev_field_ptr(t):
    """(pointer, is_bf16) of a contiguous CUDA float32 / bfloat16 tensor."""
    import torch

    if not _is_torch(t) or not t.is_cuda or not t.is_contiguous():
        raise ValueError("fields must be a contiguous CUDA tensor")
    if t.dtype == torch.bfloat16:
        return t.data_ptr(), 1
    if t.dtype == torch.float32:
        return t.data_ptr(), 0
    raise ValueError("fields must be float32 or bfloat16")


class UnaryNet:
    """The learned unary (pa_unary_net): 1x1 conv dim -> 64, three 3x3 64 -> 64
    and a 3x3 64 -> n_parts, ReLU between, BF16 operands with FP32
    accumulation on the tensor cores, FP32 master weights and Adam.  Fields
    are CUDA tensors [n][ny][nx][dim] (float32 or bfloat16)."""

    def __init__(self, ctx: Context, dim: int = 960, n_parts: int = 10, seed: int = 0):
        self.ctx, self.dim, self.P = ctx, int(dim), int(n_parts)
        h = C.c_void_p()
        ctx._check(ctx.L.pa_unary_net_create(ctx.h, self.dim, self.P, int(seed) & (2**64 - 1),
                                             C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.pa_unary_net_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_params(self) -> int:
        n = C.c_int64()
        self.ctx._check(self.ctx.L.pa_unary_net_get_params(self.ctx.h, self.h, None, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        n = C.c_int64()
        self.ctx._check(self.ctx.L.pa_unary_net_get_params(self.ctx.h, self.h,
                                                           out.ctypes.data, C.byref(n)))
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        self.ctx._check(self.ctx.L.pa_unary_net_set_params(self.ctx.h, self.h, p.ctypes.data))

    def forward(self, fields, exp_out=False, out=None):
        """Log scores (or scores with exp_out) as a CUDA tensor [P][n][ny][nx]."""
        import torch

        ptr, bf = _dev_field_ptr(fields)
        n, ny, nx, dim = fields.shape
        if dim != self.dim:
            raise ValueError("field depth differs from the net's")
        if out is None:
            out = torch.empty((self.P, n, ny, nx), dtype=torch.float32, device=fields.device)
        self.ctx._check(self.ctx.L.pa_unary_net_forward(
            self.ctx.h, self.h, ptr, bf, n, ny, nx, out.data_ptr(), ny * nx, n * ny * nx,
            int(bool(exp_out))))
        return out

    def backward(self, fields, scores, want_grads=False):
        """Loss (float) and, with want_grads, the host copy of the gradient.
        scores: CUDA float32 [P][n][ny][nx] AdaBoost score grids."""
        ptr, bf = _dev_field_ptr(fields)
        n, ny, nx, dim = fields.shape
        if tuple(scores.shape) != (self.P, n, ny, nx) or not scores.is_contiguous():
            raise ValueError("scores must be a contiguous [P][n][ny][nx] tensor")
        loss = C.c_double()
        g = np.empty(self.n_params, dtype=np.float32) if want_grads else None
        self.ctx._check(self.ctx.L.pa_unary_net_backward(
            self.ctx.h, self.h, ptr, bf, scores.data_ptr(), n, ny, nx, C.byref(loss),
            None if g is None else g.ctypes.data))
        return (loss.value, g) if want_grads else loss.value

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        a = AdamParam(float(lr), float(beta1), float(beta2), float(eps))
        self.ctx._check(self.ctx.L.pa_unary_net_adam(self.ctx.h, self.h, C.byref(a)))

    def train_step(self, fields, scores, lr=1e-3, **kw):
        loss = self.backward(fields, scores)
        self.adam(lr=lr, **kw)
        return loss


def find_obj_batch_learned(ctx: Context, exp: ExpParam, trees, net: UnaryNet, fields, Tig, H, W,
                           part_on_net=None, cls_list=None, desc=None, flip=False,
                           want_marg=False, want_root=False):
    """pa_find_obj_batch_learned: fields [B][R][ny][nx][dim] bfloat16 CUDA tensor
    (read by the net; may be None when no part is on the net), desc the float32
    descriptors for the parts off the net (may be None when every part is)."""
    ref = fields if fields is not None else desc
    if ref is None:
        raise ValueError("need the BF16 fields, the FP32 descriptors, or both")
    B, R, ny, nx, dim = ref.shape
    ths = [_TreeHolder(t) for t in trees]
    arr = (Tree * B)(*[t.s for t in ths])
    P = ths[0].s.n_parts
    T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(-1)
    results, outs = [], (PsOutputs * B)()
    for i in range(B):
        res, o = ctx._outputs(P, R, H, W, exp.roi_save_num_samples, PA_MEM_DEVICE, ref,
                              want_marg, want_root)
        results.append(res)
        outs[i] = o
    on = None
    if part_on_net is not None:
        on_arr = np.ascontiguousarray(part_on_net, dtype=np.int32)
        on = on_arr.ctypes.data
    fptr = _dev_field_ptr(fields)[0] if fields is not None else None
    dptr = _Buf(desc, np.float32).ptr if desc is not None else None
    cl = ctx._cls_array(cls_list) if cls_list else None
    ctx._check(ctx.L.pa_find_obj_batch_learned(
        ctx.h, C.byref(exp), B, arr, int(flip), net.h, on, cl, len(cls_list or []), fptr, dptr,
        ny, nx, dim, T.ctypes.data_as(C.POINTER(C.c_double)), int(T.size == 9), H, W, outs))
    return [ctx._finish(r, P) for r in results]
