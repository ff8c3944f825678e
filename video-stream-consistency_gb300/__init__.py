"""Python front end of libvsc, the GB300 (sm_103a) implementation of the
video-stream-consistency per-frame hot path.

Everything here is a thin ctypes layer over the C ABI in include/vsc.h; the
computation happens in the CUDA kernels of csrc/.  Device buffers are torch
CUDA tensors (torch provides allocation and streams only).  There is no CPU
fallback: if libvsc.so has not been built, every call raises.

Names mirror the reference interfaces they replace:
  correlation / warp          custom::Correlation / custom::Warp
                              (src/ort_custom_ops/include/ort_custom_ops/opticalflow/*.h)
  get_warp_result, get_adap_comb, get_consist_wt, get_bilinear,
  get_consist_out             src/stabilization/flowconsistency.cuh:3-50
  char_to_float_image, float_to_char_image
                              src/stabilization/gpuimage.cu:70-135
  Stabilizer                  VideoStabilizer (src/stabilization/videostabilizer.h:63-110)
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libvsc.so"

VSC_OK, VSC_EINVAL, VSC_ECUDA, VSC_ETIMEOUT, VSC_ENOMEM, VSC_EUNSUPPORTED, VSC_ESTATE = range(7)
STATUS_NAMES = ["VSC_OK", "VSC_EINVAL", "VSC_ECUDA", "VSC_ETIMEOUT", "VSC_ENOMEM", "VSC_EUNSUPPORTED", "VSC_ESTATE"]

# every symbol include/vsc.h declares (checked by the tests)
EXPORTED = [
    "vsc_last_error", "vsc_version", "vsc_correlation_fwd", "vsc_warp_fwd", "vsc_char_to_float_image",
    "vsc_float_to_char_image", "vsc_get_warp_result", "vsc_get_adap_comb", "vsc_get_consist_wt",
    "vsc_get_bilinear", "vsc_consist_out_workspace_size", "vsc_get_consist_out", "vsc_default_hyper_params",
    "vsc_stabilizer_create", "vsc_stabilizer_destroy", "vsc_stabilizer_hyper_params", "vsc_stabilizer_load_frame",
    "vsc_stabilizer_set_flows", "vsc_stabilizer_step", "vsc_stabilizer_buffer", "vsc_stabilizer_last_launches",
    "vsc_stabilizer_enable_timing", "vsc_stabilizer_stage_ms", "vsc_check_device", "vsc_selftest_bounded_wait",
    "vsc_get_consist_out_noalloc", "vsc_get_flow_consistency_mask", "vsc_get_adap_comb_masked",
    "vsc_stabilizer_set_occlusion_mask", "vsc_correlation_fwd_f64", "vsc_warp_fwd_f64",
    "vsc_correlation_lowp_workspace_size", "vsc_correlation_fwd_lowp",
    "vsc_image_file_info", "vsc_read_image_file", "vsc_write_png", "vsc_flo_info", "vsc_read_flo", "vsc_write_flo",
    "vsc_stabilize_files", "vsc_solver_steps_per_launch",
    "vsc_multistream_create", "vsc_multistream_destroy", "vsc_multistream_hyper_params", "vsc_multistream_load_frames",
    "vsc_multistream_step", "vsc_multistream_last_launches", "vsc_stab_front", "vsc_stab_front_rgba",
    "vsc_flow_estimate",
    "vsc_upsampler_param_count", "vsc_upsampler_create", "vsc_upsampler_destroy", "vsc_upsampler_get_params",
    "vsc_upsampler_set_max_residual", "vsc_upsampler_prepare", "vsc_upsampler_train_step", "vsc_upsampler_apply",
    "vsc_stabilizer_set_upsampler", "vsc_solver_autotune", "vsc_solver_tile_rows", "vsc_solver_set_autotune",
    "vsc_multistream_set_fused", "vsc_multistream_fused", "vsc_multistream_set_upsampler",
    "vsc_stabilizer_synchronize", "vsc_stabilizer_wait_output",
    "vsc_get_consist_out_fma", "vsc_consist_out_fma_workspace_size", "vsc_solver_autotune_form",
    "vsc_solver_tile_rows_form",
    "vsc_stabilizer_set_solver_form", "vsc_multistream_set_solver_form", "vsc_write_jpeg",
]
VSC_DTYPE_F32, VSC_DTYPE_BF16, VSC_DTYPE_F16 = 0, 1, 2
VSC_OUT_HOST_ASYNC = 2
NOALLOC_MAX_PIXELS = 349525  # VSC_NOALLOC_MAX_PIXELS


class VscError(RuntimeError):
    def __init__(self, status: int, message: str):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {message}")
        self.status = status


class Image(C.Structure):
    """vsc_image: interleaved float HWC device image (GPUImageWrapper)."""

    _fields_ = [("data", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("channels", C.c_int32)]


class HyperParams(C.Structure):
    """vsc_hyper_params (hyperParams, videostabilizer.h:38-46)."""

    _fields_ = [
        ("alpha", C.c_float), ("beta", C.c_float), ("gamma", C.c_float), ("pyramid_levels", C.c_int32),
        ("num_iter", C.c_int32), ("step_size", C.c_float), ("mom_fac", C.c_float),
    ]


class FilesConfig(C.Structure):
    _fields_ = [
        ("original_dir", C.c_char_p), ("processed_dir", C.c_char_p), ("output_dir", C.c_char_p),
        ("flow_dir", C.c_char_p), ("width", C.c_int32), ("height", C.c_int32), ("flow_downscale", C.c_int32),
        ("corr_dtype", C.c_int32), ("hyper", C.c_void_p), ("jpeg_quality", C.c_int32),
    ]


class StreamDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("flow_downscale", C.c_int32), ("corr_dtype", C.c_int32)]


class StabilizerConfig(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("batch_size", C.c_int32), ("compute_flow", C.c_int32),
        ("flow_downscale", C.c_int32), ("flow_channels", C.c_int32), ("use_graphs", C.c_int32),
        ("corr_dtype", C.c_int32),
    ]


_lib = None


def build(force: bool = False) -> Path:
    """Compile libvsc.so for sm_103a (see build.py)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("_vsc_build", PKG_DIR / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def load():
    """Load libvsc.so; raises if it has not been built (no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"libvsc.so not built ({LIB_PATH}); run the package build first")
    L = C.CDLL(str(LIB_PATH))
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    IP = C.POINTER(Image)
    L.vsc_last_error.restype = C.c_char_p
    L.vsc_last_error.argtypes = []
    L.vsc_version.restype = C.c_int
    for fn, args in {
        "vsc_correlation_fwd": [vp, vp, vp, i64, i64, i64, i64, i64, i64, vp],
        "vsc_warp_fwd": [vp, vp, vp, i64, i64, i64, i64, vp],
        "vsc_correlation_fwd_f64": [vp, vp, vp, i64, i64, i64, i64, i64, vp],
        "vsc_correlation_fwd_lowp": [vp, vp, vp, i64, i64, i64, i64, i64, i32, vp, C.c_size_t, vp],
        "vsc_warp_fwd_f64": [vp, vp, vp, i64, i64, i64, i64, vp],
        "vsc_char_to_float_image": [vp, IP, vp],
        "vsc_float_to_char_image": [IP, vp, vp],
        "vsc_get_warp_result": [IP, IP, IP, vp],
        "vsc_get_adap_comb": [IP] * 9 + [f32, vp],
        "vsc_get_consist_wt": [IP, IP, IP, f32, f32, vp],
        "vsc_get_bilinear": [IP, IP, vp],
        "vsc_get_consist_out": [IP, IP, IP, i32, f32, f32, IP, vp, C.c_size_t, vp],
        "vsc_get_consist_out_fma": [IP, IP, IP, i32, f32, f32, IP, vp, C.c_size_t, vp],
        "vsc_solver_autotune_form": [i32, i32, i32, vp, C.POINTER(i32)],
        "vsc_stabilizer_set_solver_form": [vp, i32],
        "vsc_multistream_set_solver_form": [vp, i32],
        "vsc_get_consist_out_noalloc": [IP, IP, IP, i32, f32, f32, IP, vp],
        "vsc_stabilizer_create": [C.POINTER(StabilizerConfig), vp, C.POINTER(vp)],
        "vsc_stabilizer_destroy": [vp],
        "vsc_stabilizer_load_frame": [vp, vp, vp, i32],
        "vsc_stabilizer_set_flows": [vp, vp, vp, i32],
        "vsc_stabilizer_step": [vp, vp, i32],
        "vsc_stabilizer_buffer": [vp, i32, C.POINTER(vp)],
        "vsc_stabilizer_enable_timing": [vp, i32],
        "vsc_get_flow_consistency_mask": [IP, IP, IP, vp],
        "vsc_stab_front": [IP] * 11 + [f32, f32, f32, i32, vp],
        "vsc_stab_front_rgba": [vp] * 6 + [IP] * 5 + [f32, f32, f32, i32, vp],
        "vsc_solver_autotune": [i32, i32, vp, C.POINTER(i32)],

        "vsc_flow_estimate": [IP, IP, IP, IP, vp],
        "vsc_upsampler_create": [vp, C.POINTER(vp)],
        "vsc_upsampler_destroy": [vp],
        "vsc_upsampler_get_params": [vp, vp],
        "vsc_upsampler_set_max_residual": [vp, f32],
        "vsc_upsampler_prepare": [IP, IP, IP, vp],
        "vsc_upsampler_train_step": [vp, vp, vp, i32, i32, i32, f32, C.POINTER(f32), vp],
        "vsc_upsampler_apply": [vp, IP, IP, IP, vp],
        "vsc_stabilizer_set_upsampler": [vp, vp],
        "vsc_image_file_info": [C.c_char_p, C.POINTER(i32), C.POINTER(i32)],
        "vsc_read_image_file": [C.c_char_p, vp, i32, i32],
        "vsc_write_png": [C.c_char_p, vp, i32, i32],
        "vsc_write_jpeg": [C.c_char_p, vp, i32, i32, i32, i32],
        "vsc_flo_info": [C.c_char_p, C.POINTER(i32), C.POINTER(i32)],
        "vsc_read_flo": [C.c_char_p, vp, i32, i32],
        "vsc_write_flo": [C.c_char_p, vp, i32, i32],
        "vsc_stabilize_files": [C.POINTER(FilesConfig), C.POINTER(i32)],
        "vsc_multistream_create": [C.POINTER(StreamDesc), i32, vp, C.POINTER(vp)],
        "vsc_multistream_destroy": [vp],
        "vsc_multistream_load_frames": [vp, C.POINTER(vp), C.POINTER(vp), i32],
        "vsc_multistream_step": [vp, C.POINTER(vp), i32],
        "vsc_multistream_set_fused": [vp, i32],
        "vsc_stabilizer_synchronize": [vp],
        "vsc_stabilizer_wait_output": [vp, i32],
        "vsc_multistream_set_upsampler": [vp, i32, vp],
        "vsc_get_adap_comb_masked": [IP] * 10 + [f32, vp],
        "vsc_stabilizer_set_occlusion_mask": [vp, i32],
        "vsc_check_device": [],
        "vsc_selftest_bounded_wait": [i32, vp],
        "vsc_stabilizer_stage_ms": [vp, C.POINTER(C.c_float), i32],
    }.items():
        f = getattr(L, fn)
        f.argtypes = args
        f.restype = C.c_int
    L.vsc_upsampler_param_count.restype = i32
    L.vsc_upsampler_param_count.argtypes = []
    L.vsc_multistream_hyper_params.restype = C.POINTER(HyperParams)
    L.vsc_multistream_hyper_params.argtypes = [vp]
    L.vsc_multistream_last_launches.restype = i32
    L.vsc_multistream_last_launches.argtypes = [vp]
    L.vsc_multistream_fused.restype = i32
    L.vsc_multistream_fused.argtypes = [vp]
    L.vsc_solver_steps_per_launch.restype = i32
    L.vsc_solver_steps_per_launch.argtypes = []
    L.vsc_solver_tile_rows.restype = i32
    L.vsc_solver_tile_rows.argtypes = [i32, i32, C.POINTER(i32)]
    L.vsc_solver_tile_rows_form.restype = i32
    L.vsc_solver_tile_rows_form.argtypes = [i32, i32, i32, C.POINTER(i32)]
    L.vsc_solver_set_autotune.restype = None
    L.vsc_solver_set_autotune.argtypes = [i32]
    L.vsc_correlation_lowp_workspace_size.restype = C.c_size_t
    L.vsc_correlation_lowp_workspace_size.argtypes = [i64, i64, i64, i64]
    L.vsc_consist_out_workspace_size.restype = C.c_size_t
    L.vsc_consist_out_workspace_size.argtypes = [i32, i32]
    L.vsc_consist_out_fma_workspace_size.restype = C.c_size_t
    L.vsc_consist_out_fma_workspace_size.argtypes = [i32, i32]
    L.vsc_default_hyper_params.restype = None
    L.vsc_default_hyper_params.argtypes = [C.POINTER(HyperParams)]
    L.vsc_stabilizer_hyper_params.restype = C.POINTER(HyperParams)
    L.vsc_stabilizer_hyper_params.argtypes = [vp]
    L.vsc_stabilizer_last_launches.restype = C.c_int32
    L.vsc_stabilizer_last_launches.argtypes = [vp]
    _lib = L
    return L


def _check(status: int) -> None:
    if status != VSC_OK:
        raise VscError(status, load().vsc_last_error().decode())


def _stream(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _f32(t, name):
    import torch

    if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
        raise ValueError(f"{name}: expected a contiguous float32 CUDA tensor")
    return t


def image(t) -> Image:
    """vsc_image view of a contiguous float32 CUDA tensor of shape (H, W, C)."""
    _f32(t, "image")
    h, w, c = t.shape
    return Image(t.data_ptr(), w, h, c)


# ---- custom ops ---------------------------------------------------------------

def _f64(t, name):
    import torch

    if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
        raise ValueError(f"{name}: expected a contiguous float64 CUDA tensor")


def correlation(f1, f2, max_displacement: int = 4, legacy: int = 0, out=None, stream=None):
    """custom::Correlation on N x C x H x W float (or, like the reference's
    CPU kernel, double) tensors."""
    import torch

    N, Cc, H, W = f1.shape
    P = 2 * max_displacement + 1
    if f1.dtype == torch.float64:
        if legacy:
            raise ValueError("correlation: the legacy form has no double version (correlation.h:45-46)")
        _f64(f1, "f1")
        _f64(f2, "f2")
        if out is None:
            out = torch.empty((N, P, P, H, W), dtype=torch.float64, device=f1.device)
        _check(load().vsc_correlation_fwd_f64(f1.data_ptr(), f2.data_ptr(), out.data_ptr(), N, Cc, H, W,
                                              max_displacement, _stream(stream)))
        return out
    _f32(f1, "f1")
    _f32(f2, "f2")
    shape = (N, P * P, H, W) if legacy else (N, P, P, H, W)
    if out is None:
        out = torch.empty(shape, dtype=torch.float32, device=f1.device)
    _check(load().vsc_correlation_fwd(f1.data_ptr(), f2.data_ptr(), out.data_ptr(), N, Cc, H, W,
                                      max_displacement, legacy, _stream(stream)))
    return out


def correlation_lowp(f1, f2, max_displacement: int = 4, dtype: str = "bf16", out=None, workspace=None,
                     stream=None):
    """custom::Correlation (legacy 0 layout) on the tensor cores with BF16 or
    FP16 operands and FP32 accumulation; f1, f2 float32 N x C x H x W."""
    import torch

    _f32(f1, "f1")
    _f32(f2, "f2")
    N, Cc, H, W = f1.shape
    P = 2 * max_displacement + 1
    if out is None:
        out = torch.empty((N, P, P, H, W), dtype=torch.float32, device=f1.device)
    code = {"bf16": VSC_DTYPE_BF16, "fp16": VSC_DTYPE_F16, "f16": VSC_DTYPE_F16}[dtype]
    ws_ptr, ws_bytes = (None, 0) if workspace is None else (workspace.data_ptr(),
                                                           workspace.numel() * workspace.element_size())
    _check(load().vsc_correlation_fwd_lowp(f1.data_ptr(), f2.data_ptr(), out.data_ptr(), N, Cc, H, W,
                                           max_displacement, code, ws_ptr, ws_bytes, _stream(stream)))
    return out


def warp(x, flow, out=None, stream=None):
    """custom::Warp: x N x C x H x W, flow N x 2 x H x W (float, or double)."""
    import torch

    N, Cc, H, W = x.shape
    if out is None:
        out = torch.empty_like(x)
    if x.dtype == torch.float64:
        _f64(x, "input")
        _f64(flow, "flow")
        _check(load().vsc_warp_fwd_f64(x.data_ptr(), flow.data_ptr(), out.data_ptr(), N, Cc, H, W,
                                       _stream(stream)))
        return out
    _f32(x, "input")
    _f32(flow, "flow")
    _check(load().vsc_warp_fwd(x.data_ptr(), flow.data_ptr(), out.data_ptr(), N, Cc, H, W, _stream(stream)))
    return out


# ---- stabilization kernels ----------------------------------------------------

def char_to_float_image(rgba, stream=None):
    import torch

    h, w = rgba.shape[:2]
    out = torch.empty((h, w, 3), dtype=torch.float32, device=rgba.device)
    _check(load().vsc_char_to_float_image(rgba.data_ptr(), C.byref(image(out)), _stream(stream)))
    return out


def float_to_char_image(img, stream=None):
    import torch

    h, w = img.shape[:2]
    out = torch.empty((h, w, 4), dtype=torch.uint8, device=img.device)
    _check(load().vsc_float_to_char_image(C.byref(image(img)), out.data_ptr(), _stream(stream)))
    return out


def get_warp_result(inp, flow, stream=None):
    import torch

    out = torch.empty_like(inp)
    _check(load().vsc_get_warp_result(C.byref(image(inp)), C.byref(image(flow)), C.byref(image(out)),
                                      _stream(stream)))
    return out


def get_adap_comb(crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr, last_stab_warp, alpha, stream=None):
    import torch

    ain = torch.empty_like(crnt_in)
    apr = torch.empty_like(crnt_in)
    ims = [image(t) for t in (crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr, ain, apr, last_stab_warp)]
    _check(load().vsc_get_adap_comb(*[C.byref(i) for i in ims], float(alpha), _stream(stream)))
    return ain, apr


def get_flow_consistency_mask(flow_fwd, flow_bwd, stream=None):
    """Forward-backward flow consistency mask (opt-in extension): HWC2 of 0/1,
    ch0 for the previous frame's warp, ch1 for the next frame's."""
    import torch

    h, w = flow_fwd.shape[:2]
    mask = torch.empty((h, w, 2), dtype=torch.float32, device=flow_fwd.device)
    _check(load().vsc_get_flow_consistency_mask(C.byref(image(flow_fwd)), C.byref(image(flow_bwd)),
                                                C.byref(image(mask)), _stream(stream)))
    return mask


def get_adap_comb_masked(crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr, last_stab_warp, occ_mask, alpha,
                         stream=None):
    """get_adap_comb with the temporal weights multiplied by occ_mask (HWC2)."""
    import torch

    ain = torch.empty_like(crnt_in)
    apr = torch.empty_like(crnt_in)
    ims = [image(t) for t in (crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr, ain, apr, last_stab_warp,
                              occ_mask)]
    _check(load().vsc_get_adap_comb_masked(*[C.byref(i) for i in ims], float(alpha), _stream(stream)))
    return ain, apr


def flow_estimate(img_a, img_b, stream=None):
    """Forward and backward flow (HWC3 (u, v, 0)) of two float HWC3 frames."""
    import torch

    ab, ba = torch.empty_like(img_a), torch.empty_like(img_a)
    _check(load().vsc_flow_estimate(C.byref(image(img_a)), C.byref(image(img_b)), C.byref(image(ab)),
                                    C.byref(image(ba)), _stream(stream)))
    return ab, ba


def stab_front(orig3, proc3, last_stab, flow_fwd, flow_bwd, alpha, beta, gamma, occlusion_mask=False, out=None,
               stream=None):
    """Five warps + adaptive combination + consistency weights in one pass;
    returns (adapCmbPr, consWt)."""
    import torch

    apr, wt = out if out is not None else (torch.empty_like(orig3[1]), torch.empty_like(orig3[1]))
    ims = [image(t) for t in (*orig3, *proc3, last_stab, flow_fwd, flow_bwd, apr, wt)]
    _check(load().vsc_stab_front(*[C.byref(i) for i in ims], float(alpha), float(beta), float(gamma),
                                 1 if occlusion_mask else 0, _stream(stream)))
    return apr, wt


def stab_front_rgba(orig3, proc3, last_stab, flow_fwd, flow_bwd, alpha, beta, gamma, occlusion_mask=False,
                    out=None, stream=None):
    """stab_front with the six frames as (h, w, 4) uint8 RGBA device tensors;
    returns (adapCmbPr, consWt), equal bit for bit to stab_front on the
    frames converted by char_to_float_image."""
    import torch

    frames = [*orig3, *proc3]
    for f in frames:
        if f.dtype != torch.uint8 or f.dim() != 3 or f.shape[2] != 4 or not f.is_contiguous() or not f.is_cuda:
            raise ValueError("stab_front_rgba: frames must be contiguous (h, w, 4) uint8 CUDA tensors")
    if out is None:
        h, w = last_stab.shape[:2]
        out = (torch.empty((h, w, 3), dtype=torch.float32, device=last_stab.device),
               torch.empty((h, w, 3), dtype=torch.float32, device=last_stab.device))
    apr, wt = out
    ims = [image(t) for t in (last_stab, flow_fwd, flow_bwd, apr, wt)]
    _check(load().vsc_stab_front_rgba(*[C.c_void_p(f.data_ptr()) for f in frames], *[C.byref(i) for i in ims],
                                      float(alpha), float(beta), float(gamma), 1 if occlusion_mask else 0,
                                      _stream(stream)))
    return apr, wt


def get_consist_wt(adap_in, crnt_in, beta, gamma, stream=None):
    import torch

    out = torch.empty_like(crnt_in)
    _check(load().vsc_get_consist_wt(C.byref(image(adap_in)), C.byref(image(crnt_in)), C.byref(image(out)),
                                     float(beta), float(gamma), _stream(stream)))
    return out


def get_bilinear(inp, ow: int, oh: int, stream=None):
    import torch

    out = torch.empty((oh, ow, inp.shape[2]), dtype=torch.float32, device=inp.device)
    _check(load().vsc_get_bilinear(C.byref(image(inp)), C.byref(image(out)), _stream(stream)))
    return out


SOLVER_FORMS = {"exact": 0, "fma": 1}  # VSC_SOLVER_EXACT, VSC_SOLVER_FMA


def solver_autotune(w: int, h: int, stream=None, form: str = "exact") -> int:
    """Time both tile shapes of the exact solver form at w x h and keep the
    faster; returns its rows (exact: 32 or 48; the fma form has one, 72)."""
    rows = C.c_int32()
    _check(load().vsc_solver_autotune_form(int(w), int(h), SOLVER_FORMS[form], _stream(stream), C.byref(rows)))
    return rows.value


def solver_tile_rows(w: int, h: int, form: str = "exact"):
    """(rows, tuned): the tile rows a solve at w x h uses, and whether they were measured."""
    tuned = C.c_int32()
    rows = load().vsc_solver_tile_rows_form(int(w), int(h), SOLVER_FORMS[form], C.byref(tuned))
    return rows, bool(tuned.value)


def solver_set_autotune(on: bool) -> None:
    load().vsc_solver_set_autotune(1 if on else 0)


def consist_out_workspace_size(w: int, h: int, form: str = "exact") -> int:
    fn = load().vsc_consist_out_fma_workspace_size if form == "fma" else load().vsc_consist_out_workspace_size
    return int(fn(w, h))


def get_consist_out(crnt_pr, prev_stab_warp, cons_wt, num_iter, step_size, mom_fac, consis_out, workspace=None,
                    stream=None, form: str = "exact"):
    """In place on consis_out (initial solution in, result out); form
    "exact" (vsc_get_consist_out) or "fma" (vsc_get_consist_out_fma)."""
    ws = workspace.data_ptr() if workspace is not None else None
    nbytes = workspace.numel() * workspace.element_size() if workspace is not None else 0
    fn = {"exact": load().vsc_get_consist_out, "fma": load().vsc_get_consist_out_fma}[form]
    _check(fn(C.byref(image(crnt_pr)), C.byref(image(prev_stab_warp)), C.byref(image(cons_wt)), int(num_iter),
              float(step_size), float(mom_fac), C.byref(image(consis_out)), ws, nbytes, _stream(stream)))
    return consis_out


def check_device() -> None:
    """Raises VscError(VSC_ETIMEOUT) if a kernel's bounded wait gave up."""
    _check(load().vsc_check_device())


def get_consist_out_noalloc(crnt_pr, prev_stab_warp, cons_wt, num_iter, step_size, mom_fac, consis_out,
                            stream=None):
    """get_consist_out with the library's built-in workspace: no device memory
    is allocated (images up to NOALLOC_MAX_PIXELS pixels; calls must not
    overlap on the GPU)."""
    _check(load().vsc_get_consist_out_noalloc(C.byref(image(crnt_pr)), C.byref(image(prev_stab_warp)),
                                              C.byref(image(cons_wt)), int(num_iter), float(step_size),
                                              float(mom_fac), C.byref(image(consis_out)), _stream(stream)))
    return consis_out


# ---- files ----------------------------------------------------------------------

def read_image(path):
    """RGBA8 numpy array of a PNG / PPM / JPEG file."""
    import numpy as np

    w, h = C.c_int32(), C.c_int32()
    _check(load().vsc_image_file_info(str(path).encode(), C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value, 4), np.uint8)
    _check(load().vsc_read_image_file(str(path).encode(), out.ctypes.data, w.value, h.value))
    return out


def write_png(path, rgba):
    import numpy as np

    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    _check(load().vsc_write_png(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0]))


def write_jpeg(path, rgba, quality: int = 75, chroma_444: bool = False, restart_rows: bool = False,
               grey: bool = False):
    """Baseline JFIF JPEG of an RGBA8 array (alpha ignored)."""
    import numpy as np

    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    flags = (1 if chroma_444 else 0) | (2 if restart_rows else 0) | (4 if grey else 0)
    _check(load().vsc_write_jpeg(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0], int(quality), flags))


def read_flo(path):
    import numpy as np

    w, h = C.c_int32(), C.c_int32()
    _check(load().vsc_flo_info(str(path).encode(), C.byref(w), C.byref(h)))
    out = np.empty((h.value, w.value, 2), np.float32)
    _check(load().vsc_read_flo(str(path).encode(), out.ctypes.data, w.value, h.value))
    return out


def write_flo(path, flow):
    import numpy as np

    a = np.ascontiguousarray(flow, dtype=np.float32)
    _check(load().vsc_write_flo(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0]))


def stabilize_files(original_dir, processed_dir, output_dir, flow_dir=None, width=0, height=0, flow_downscale=1,
                    corr_dtype: str = "f32", hyper: "HyperParams | None" = None, jpeg_quality: int = 0) -> int:
    """Headless FileStabilizer: stabilizes a frame directory; returns the number
    of frames written (PNG files, or .jpg at jpeg_quality 1..100)."""
    code = {"f32": VSC_DTYPE_F32, "bf16": VSC_DTYPE_BF16, "fp16": VSC_DTYPE_F16}[corr_dtype]
    cfg = FilesConfig(str(original_dir).encode(), str(processed_dir).encode(), str(output_dir).encode(),
                      str(flow_dir).encode() if flow_dir else None, width, height, flow_downscale, code,
                      C.cast(C.pointer(hyper), C.c_void_p) if hyper is not None else None, int(jpeg_quality))
    n = C.c_int32()
    _check(load().vsc_stabilize_files(C.byref(cfg), C.byref(n)))
    return n.value


def default_hyper_params() -> HyperParams:
    hp = HyperParams()
    load().vsc_default_hyper_params(C.byref(hp))
    return hp


class _DeviceView:
    """Zero-copy view of library-owned device memory (float32), for torch.as_tensor."""

    def __init__(self, ptr: int, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f4", "data": (ptr, False),
                                         "version": 3, "strides": None}


class Stabilizer:
    """VideoStabilizer without Qt: feed RGBA frames, get stabilized RGBA frames.

    compute_flow=True computes flows with the library's estimator (built on
    the Correlation and Warp kernels); otherwise call set_flows before each
    step.
    """

    def __init__(self, width, height, compute_flow=True, flow_downscale=1, flow_channels=3, stream=None,
                 use_graphs=True, corr_dtype: str = "f32", solver_form: str = "exact"):
        """corr_dtype: "f32" (the plain method), "bf16" or "fp16" (the flow
        estimator's correlations on the tensor cores); solver_form: "exact"
        (the reference's arithmetic) or "fma" (vsc_stabilizer_set_solver_form)."""
        import torch

        self.width, self.height = width, height
        self._stream_obj = stream if stream is not None else torch.cuda.current_stream()
        code = {"f32": VSC_DTYPE_F32, "bf16": VSC_DTYPE_BF16, "fp16": VSC_DTYPE_F16, "f16": VSC_DTYPE_F16}[corr_dtype]
        cfg = StabilizerConfig(width, height, 1, 1 if compute_flow else 0, flow_downscale, flow_channels,
                               1 if use_graphs else 0, code)
        h = C.c_void_p()
        _check(load().vsc_stabilizer_create(C.byref(cfg), _stream(self._stream_obj), C.byref(h)))
        self._h = h
        if solver_form != "exact":
            self.set_solver_form(solver_form)

    def set_solver_form(self, form: str):
        """"exact" or "fma": the blend solver's form for the following steps."""
        _check(load().vsc_stabilizer_set_solver_form(self._h, SOLVER_FORMS[form]))

    @property
    def hyper_params(self) -> HyperParams:
        return load().vsc_stabilizer_hyper_params(self._h).contents

    def load_frame(self, orig_rgba, proc_rgba):
        """orig/proc: uint8 (H, W, 4) tensors on the device, or numpy arrays / CPU tensors."""
        import numpy as np

        on_dev = 1 if getattr(orig_rgba, "is_cuda", False) else 0
        if on_dev:
            a, b = orig_rgba.data_ptr(), proc_rgba.data_ptr()
        else:
            oa = np.ascontiguousarray(orig_rgba if isinstance(orig_rgba, np.ndarray) else orig_rgba.numpy())
            pa = np.ascontiguousarray(proc_rgba if isinstance(proc_rgba, np.ndarray) else proc_rgba.numpy())
            self._keep = (oa, pa)
            a, b = oa.ctypes.data, pa.ctypes.data
        _check(load().vsc_stabilizer_load_frame(self._h, a, b, on_dev))

    def set_flows(self, fwd, bwd):
        _check(load().vsc_stabilizer_set_flows(self._h, fwd.data_ptr(), bwd.data_ptr(), 1 if fwd.is_cuda else 0))

    def step(self, out=None, asynchronous: bool = False):
        """Stabilize the window's middle frame; returns the RGBA result.  With
        a host tensor and asynchronous=True the copy back is only enqueued
        (VSC_OUT_HOST_ASYNC): read `out` after wait_output() or synchronize()."""
        import torch

        if out is None:
            out = torch.empty((self.height, self.width, 4), dtype=torch.uint8, device="cuda")
        mode = 1 if out.is_cuda else (VSC_OUT_HOST_ASYNC if asynchronous else 0)
        _check(load().vsc_stabilizer_step(self._h, out.data_ptr(), mode))
        return out

    def synchronize(self):
        _check(load().vsc_stabilizer_synchronize(self._h))

    def wait_output(self, which: int = 0):
        """Waits for the host copy of the last asynchronous step (0) or the one before (1)."""
        _check(load().vsc_stabilizer_wait_output(self._h, which))

    def buffer(self, which: int, channels: int = 3):
        """Copy of internal state: 0 last stabilized, 1 fwd flow, 2 bwd flow, 3 adapCmbPr, 4 consWt."""
        import torch

        p = C.c_void_p()
        _check(load().vsc_stabilizer_buffer(self._h, which, C.byref(p)))
        self._stream_obj.synchronize()
        view = _DeviceView(p.value, (self.height, self.width, channels))
        return torch.as_tensor(view, device="cuda").clone()

    STAGES = ("load", "flow", "front", "coarse_solve", "full_solve")

    def set_occlusion_mask(self, on: bool = True):
        """Opt-in forward-backward flow consistency mask on the temporal weights."""
        _check(load().vsc_stabilizer_set_occlusion_mask(self._h, 1 if on else 0))

    def set_upsampler(self, upsampler: "Upsampler | None"):
        """Learned flow upsampling (flow_downscale > 1); None: bilinear.  The
        stabilizer keeps a reference for as long as it uses it."""
        self._upsampler = upsampler
        _check(load().vsc_stabilizer_set_upsampler(self._h, upsampler._h if upsampler is not None else None))

    def enable_timing(self, on: bool = True):
        _check(load().vsc_stabilizer_enable_timing(self._h, 1 if on else 0))

    def stage_ms(self) -> dict:
        """Device time of the stages of the last load_frame and step (ms)."""
        buf = (C.c_float * 5)()
        _check(load().vsc_stabilizer_stage_ms(self._h, buf, 5))
        return dict(zip(self.STAGES, list(buf)))

    @property
    def last_launches(self) -> int:
        return int(load().vsc_stabilizer_last_launches(self._h))

    def close(self):
        if getattr(self, "_h", None):
            load().vsc_stabilizer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultiStream:
    """Several independent videos stabilized in lockstep, one graph launch per
    frame step, the solves of all videos grouped into shared launches of the
    persistent solver kernel (vsc_multistream_*).  sizes: [(width, height),
    ...]; flow_downscale and corr_dtype: one value for every stream or a
    list with one per stream."""

    def __init__(self, sizes, flow_downscale=1, corr_dtype="f32", stream=None):
        import torch

        codes = {"f32": VSC_DTYPE_F32, "bf16": VSC_DTYPE_BF16, "fp16": VSC_DTYPE_F16}
        self.sizes = [tuple(x) for x in sizes]
        n = len(self.sizes)
        ds = list(flow_downscale) if isinstance(flow_downscale, (list, tuple)) else [flow_downscale] * n
        dt = list(corr_dtype) if isinstance(corr_dtype, (list, tuple)) else [corr_dtype] * n
        if len(ds) != n or len(dt) != n:
            raise ValueError("one flow_downscale and corr_dtype per stream")
        descs = (StreamDesc * n)(*[StreamDesc(w, h, d, codes[c]) for (w, h), d, c in zip(self.sizes, ds, dt)])
        self._stream_obj = stream if stream is not None else torch.cuda.current_stream()
        h = C.c_void_p()
        _check(load().vsc_multistream_create(descs, n, _stream(self._stream_obj), C.byref(h)))
        self._h = h
        self._upsamplers = {}

    @property
    def hyper_params(self) -> HyperParams:
        return load().vsc_multistream_hyper_params(self._h).contents

    @property
    def last_launches(self) -> int:
        return int(load().vsc_multistream_last_launches(self._h))

    @property
    def fused(self) -> bool:
        """True when a step with the current hyper-parameters groups the solves."""
        return bool(load().vsc_multistream_fused(self._h))

    def set_fused(self, on: bool):
        _check(load().vsc_multistream_set_fused(self._h, 1 if on else 0))

    def set_solver_form(self, form: str):
        """"exact" or "fma" for every stream's solves."""
        _check(load().vsc_multistream_set_solver_form(self._h, SOLVER_FORMS[form]))

    def set_upsampler(self, upsampler, index: int = -1):
        """The learned upsampler for stream `index` (-1: every stream with
        flow_downscale > 1); None: bilinear."""
        _check(load().vsc_multistream_set_upsampler(self._h, index, upsampler._h if upsampler else None))
        self._upsamplers[index] = upsampler  # kept alive while the streams use it

    def load_frames(self, origs, procs):
        """One RGBA8 (H, W, 4) frame pair per stream: all numpy (host) or all CUDA tensors."""
        import numpy as np

        on_dev = hasattr(origs[0], "is_cuda") and origs[0].is_cuda
        keep = []

        def ptr(a):
            if on_dev:
                return a.data_ptr()
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data

        o = (C.c_void_p * len(origs))(*[ptr(a) for a in origs])
        p = (C.c_void_p * len(procs))(*[ptr(a) for a in procs])
        _check(load().vsc_multistream_load_frames(self._h, o, p, 1 if on_dev else 0))

    def step(self, outs=None):
        """Stabilizes every stream's middle frame; returns the RGBA8 results
        (device tensors unless host arrays are given)."""
        import torch

        if outs is None:
            outs = [torch.empty((h, w, 4), dtype=torch.uint8, device="cuda") for w, h in self.sizes]
        on_dev = hasattr(outs[0], "is_cuda") and outs[0].is_cuda
        ptrs = (C.c_void_p * len(outs))(*[(o.data_ptr() if on_dev else o.ctypes.data) for o in outs])
        _check(load().vsc_multistream_step(self._h, ptrs, 1 if on_dev else 0))
        return outs

    def close(self):
        if getattr(self, "_h", None):
            load().vsc_multistream_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


UPSAMPLER_WEIGHTS = PKG_DIR / "upsampler_weights.npz"


class Upsampler:
    """Learned 2x flow upsampler (vsc_upsampler_*): params None for the
    seeded initialisation, "default" for the weights shipped with the
    package, or an array of vsc_upsampler_param_count floats."""

    def __init__(self, params=None):
        import numpy as np

        if isinstance(params, str) and params == "default":
            params = np.load(UPSAMPLER_WEIGHTS)["params"]
        arr = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        if arr is not None and arr.size != self.param_count():
            raise ValueError(f"expected {self.param_count()} parameters, got {arr.size}")
        h = C.c_void_p()
        _check(load().vsc_upsampler_create(None if arr is None else arr.ctypes.data, C.byref(h)))
        self._h = h

    @staticmethod
    def param_count() -> int:
        return int(load().vsc_upsampler_param_count())

    def params(self):
        import numpy as np

        out = np.empty(self.param_count(), np.float32)
        _check(load().vsc_upsampler_get_params(self._h, out.ctypes.data))
        return out

    def set_max_residual(self, px: float):
        _check(load().vsc_upsampler_set_max_residual(self._h, float(px)))

    @staticmethod
    def prepare(coarse_flow, frame, stream=None):
        """(h, w, 3) input: base flow (bilinear, vectors scaled) and luma."""
        import torch

        out = torch.empty_like(frame)
        _check(load().vsc_upsampler_prepare(C.byref(image(coarse_flow)), C.byref(image(frame)), C.byref(image(out)),
                                            _stream(stream)))
        return out

    def train_step(self, inputs, targets, lr: float, stream=None) -> float:
        """inputs (n, h, w, 3), targets (n, h, w, 2): CUDA float32; returns the batch loss."""
        n, h, w, _ = inputs.shape
        loss = C.c_float()
        _check(load().vsc_upsampler_train_step(self._h, inputs.data_ptr(), targets.data_ptr(), n, h, w, float(lr),
                                               C.byref(loss), _stream(stream)))
        return loss.value

    def apply(self, coarse_flow, frame, stream=None):
        import torch

        out = torch.empty_like(frame)
        _check(load().vsc_upsampler_apply(self._h, C.byref(image(coarse_flow)), C.byref(image(frame)),
                                          C.byref(image(out)), _stream(stream)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            load().vsc_upsampler_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

