"""ctypes front end of the checker (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (the C restatement of the reference's hot
path, ``vsc_oracle.c``) and, where it was built, ``oracle/_ref/libref_ops.so``
(the reference's own CPU custom ops compiled in place).  Only tests, the smoke
check and bench.py's CPU-baseline leg import this module; the product library
never does.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_PATH = HERE / "_ref" / "libref_ops.so"

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i = C.c_int
_i64 = C.c_int64


class Hyper(C.Structure):
    """Mirror of vo_hyper / the reference's hyperParams (videostabilizer.h:38-46)."""

    _fields_ = [
        ("alpha", C.c_float),
        ("beta", C.c_float),
        ("gamma", C.c_float),
        ("pyramid_levels", C.c_int),
        ("num_iter", C.c_int),
        ("step_size", C.c_float),
        ("mom_fac", C.c_float),
    ]


def build(ref: bool = True) -> None:
    """Compile the restatement (and the in-place reference ops when the
    reference tree is present)."""
    targets = ["_build/liboracle.so"]
    if shutil.which("nvcc") or Path("/usr/local/cuda/bin/nvcc").exists():
        targets.append("_build/librefgpu.so")
    subprocess.run(["make", "-s", "-C", str(HERE), *targets], check=True)
    # the reference checkout: VSC_REFERENCE_ROOT, else "reference" beside this checkout
    refdir = os.environ.get("VSC_REFERENCE_ROOT", str(HERE.parent.parent / "reference"))
    if ref and Path(refdir, "src", "ort_custom_ops").is_dir():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", "refgpu", f"REF={refdir}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build(ref=False)
        L = C.CDLL(str(LIB_PATH))
        L.vo_expf.restype = C.c_float
        L.vo_expf.argtypes = [C.c_float]
        L.vo_set_threads.argtypes = [_i]
        L.vo_get_threads.restype = _i
        L.vo_correlation_f32.argtypes = [_f32p, _f32p, _f32p, _i, _i, _i, _i, _i]
        L.vo_correlation_f64.argtypes = [_f64p, _f64p, _f64p, _i, _i, _i, _i, _i]
        L.vo_correlation_legacy_f32.argtypes = [_f32p, _f32p, _f32p, _i, _i, _i, _i, _i]
        for fn in ("vo_warp_op_refsem", "vo_warp_op_f32"):
            getattr(L, fn).argtypes = [_f32p, _f32p, _f32p, _i, _i, _i, _i]
        L.vo_warp_op_f64.argtypes = [_f64p, _f64p, _f64p, _i, _i, _i, _i]
        L.vo_rgba_to_float.argtypes = [_u8p, _f32p, _i64]
        L.vo_float_to_rgba.argtypes = [_f32p, _u8p, _i64]
        L.vo_stab_warp.argtypes = [_f32p, _f32p, _i, _f32p, _i, _i]
        L.vo_adap_comb.argtypes = [_f32p] * 9 + [C.c_float, _i64]
        L.vo_adap_comb_masked.argtypes = [_f32p] * 9 + [C.c_void_p, C.c_float, _i64]
        L.vo_flow_consistency_mask.argtypes = [_f32p, _f32p, _i, _f32p, _i, _i]
        L.vo_consist_wt.argtypes = [_f32p, _f32p, _f32p, C.c_float, C.c_float, _i64]
        L.vo_bilinear.argtypes = [_f32p, _i, _i, _f32p, _i, _i, _i]
        L.vo_consist_out.argtypes = [_f32p, _f32p, _f32p, _i, C.c_float, C.c_float, _f32p, _i, _i]
        L.vo_consist_out_fma.argtypes = [_f32p, _f32p, _f32p, _i, C.c_float, C.c_float, _f32p, _i, _i]
        L.vo_default_hyper.argtypes = [C.POINTER(Hyper)]
        L.vo_stab_pass.restype = _i
        L.vo_stab_pass.argtypes = [
            _i, _i, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _f32p, _f32p, _i, _f32p,
            C.POINTER(Hyper), _f32p, C.c_void_p,
        ]
        L.vo_stab_pass_ex.restype = _i
        L.vo_stab_pass_ex.argtypes = [
            _i, _i, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _f32p, _f32p, _i, _f32p,
            C.POINTER(Hyper), _i, _f32p, C.c_void_p,
        ]
        L.vo_stab_pass_form.restype = _i
        L.vo_stab_pass_form.argtypes = [
            _i, _i, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), _f32p, _f32p, _i, _f32p,
            C.POINTER(Hyper), _i, _i, _f32p, C.c_void_p,
        ]
        L.vo_flow_level_dims.argtypes = [_i, _i, _i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)]
        L.vo_flow_feature_floats.restype = C.c_size_t
        L.vo_flow_feature_floats.argtypes = [_i, _i]
        L.vo_flow_weights.argtypes = [_i, _f32p]
        L.vo_flow_features.argtypes = [_f32p, _i, _i, _f32p]
        L.vo_flow_from_features.argtypes = [_f32p, _f32p, _i, _i, _f32p]
        L.vo_flow_estimate.argtypes = [_f32p, _f32p, _i, _i, _f32p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return REF_PATH.exists()


def ref():
    """The reference's own CPU custom ops (correlation.cc, warp.cc), or None."""
    global _ref
    if _ref is None and REF_PATH.exists():
        R = C.CDLL(str(REF_PATH))
        R.ref_last_error.restype = C.c_char_p
        R.ref_correlation_f32.argtypes = [_f32p, _f32p, _f32p] + [_i64] * 6
        R.ref_correlation_f64.argtypes = [_f64p, _f64p, _f64p] + [_i64] * 6
        R.ref_warp_f32.argtypes = [_f32p, _f32p, _f32p] + [_i64] * 4
        R.ref_warp_f64.argtypes = [_f64p, _f64p, _f64p] + [_i64] * 4
        for fn in ("ref_correlation_f32", "ref_correlation_f64", "ref_warp_f32", "ref_warp_f64"):
            getattr(R, fn).restype = C.c_int
        _ref = R
    return _ref


def set_threads(n: int) -> None:
    lib().vo_set_threads(int(n))


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---- ops -------------------------------------------------------------------

def correlation(f1, f2, md: int = 4, legacy: int = 0):
    dt = np.float64 if np.asarray(f1).dtype == np.float64 else np.float32
    f1 = _c(f1, dt)
    f2 = _c(f2, dt)
    N, Cc, H, W = f1.shape
    P = 2 * md + 1
    if legacy:
        out = np.empty((N, P * P, H, W), np.float32)
        lib().vo_correlation_legacy_f32(f1, f2, out, N, Cc, H, W, md)
        return out
    out = np.empty((N, P, P, H, W), dt)
    fn = lib().vo_correlation_f64 if dt == np.float64 else lib().vo_correlation_f32
    fn(f1, f2, out, N, Cc, H, W, md)
    return out


def warp_op(x, flow, form: str = "f32"):
    """form: 'f32' (the GPU's single-precision arithmetic), 'refsem' (the
    reference's double-precision weights, bit-exact to warp.cc) or 'f64'."""
    if form == "f64":
        x = _c(x, np.float64)
        flow = _c(flow, np.float64)
        out = np.empty_like(x)
        lib().vo_warp_op_f64(x, flow, out, *x.shape)
        return out
    x = _c(x, np.float32)
    flow = _c(flow, np.float32)
    out = np.empty_like(x)
    fn = lib().vo_warp_op_refsem if form == "refsem" else lib().vo_warp_op_f32
    fn(x, flow, out, *x.shape)
    return out


def ref_correlation(f1, f2, md: int = 4, legacy: int = 0):
    R = ref()
    dt = np.float64 if np.asarray(f1).dtype == np.float64 else np.float32
    f1 = _c(f1, dt)
    f2 = _c(f2, dt)
    N, Cc, H, W = f1.shape
    P = 2 * md + 1
    out = np.empty((N, P, P, H, W), dt)
    fn = R.ref_correlation_f64 if dt == np.float64 else R.ref_correlation_f32
    rc = fn(f1, f2, out, N, Cc, H, W, md, legacy)
    if rc != 0:
        raise RuntimeError(R.ref_last_error().decode())
    return out


def ref_warp(x, flow):
    R = ref()
    dt = np.float64 if np.asarray(x).dtype == np.float64 else np.float32
    x = _c(x, dt)
    flow = _c(flow, dt)
    out = np.empty_like(x)
    fn = R.ref_warp_f64 if dt == np.float64 else R.ref_warp_f32
    rc = fn(x, flow, out, *x.shape)
    if rc != 0:
        raise RuntimeError(R.ref_last_error().decode())
    return out


# ---- frame I/O and stabilization ---------------------------------------------

def rgba_to_float(rgba):
    rgba = _c(rgba, np.uint8)
    h, w = rgba.shape[:2]
    out = np.empty((h, w, 3), np.float32)
    lib().vo_rgba_to_float(rgba, out, h * w)
    return out


def float_to_rgba(img):
    img = _c(img, np.float32)
    h, w = img.shape[:2]
    out = np.empty((h, w, 4), np.uint8)
    lib().vo_float_to_rgba(img, out, h * w)
    return out


def stab_warp(img, flow):
    img = _c(img, np.float32)
    flow = _c(flow, np.float32)
    h, w = img.shape[:2]
    out = np.empty_like(img)
    lib().vo_stab_warp(img, flow, flow.shape[2], out, w, h)
    return out


def adap_comb(crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr, last_stab_warp, alpha):
    args = [_c(a, np.float32) for a in (crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr)]
    ain = np.empty_like(args[0])
    apr = np.empty_like(args[0])
    npix = args[0].shape[0] * args[0].shape[1]
    lib().vo_adap_comb(*args, ain, apr, _c(last_stab_warp, np.float32), float(alpha), npix)
    return ain, apr


def adap_comb_masked(crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr, last_stab_warp, occ_mask, alpha):
    """adap_comb with the temporal weights multiplied by occ_mask (HWC2: previous, next)."""
    args = [_c(a, np.float32) for a in (crnt_in, crnt_pr, prev_in, prev_pr, next_in, next_pr)]
    ain = np.empty_like(args[0])
    apr = np.empty_like(args[0])
    npix = args[0].shape[0] * args[0].shape[1]
    m = _c(occ_mask, np.float32)
    lib().vo_adap_comb_masked(*args, ain, apr, _c(last_stab_warp, np.float32), m.ctypes.data, float(alpha), npix)
    return ain, apr


def flow_consistency_mask(flow_fwd, flow_bwd):
    """Forward-backward consistency mask, HWC2 of 0/1 (ch0 previous, ch1 next)."""
    ff = _c(flow_fwd, np.float32)
    fb = _c(flow_bwd, np.float32)
    h, w, fc = ff.shape
    out = np.empty((h, w, 2), np.float32)
    lib().vo_flow_consistency_mask(ff, fb, fc, out, w, h)
    return out


def consist_wt(crnt_in, adap_in, beta, gamma):
    ci = _c(crnt_in, np.float32)
    out = np.empty_like(ci)
    lib().vo_consist_wt(ci, _c(adap_in, np.float32), out, float(beta), float(gamma), ci.shape[0] * ci.shape[1])
    return out


def bilinear(img, ow: int, oh: int):
    img = _c(img, np.float32)
    ih, iw, c = img.shape
    out = np.empty((oh, ow, c), np.float32)
    lib().vo_bilinear(img, iw, ih, out, ow, oh, c)
    return out


def consist_out(P, A, wt, num_iter, step, mom, O_init, form: str = "exact"):
    """form: 'exact' (kernel_consist_out's expression) or 'fma' (the
    library's FMA form of the same iteration)."""
    O = _c(O_init, np.float32).copy()
    h, w = O.shape[:2]
    fn = lib().vo_consist_out_fma if form == "fma" else lib().vo_consist_out
    fn(_c(P, np.float32), _c(A, np.float32), _c(wt, np.float32), int(num_iter), float(step), float(mom), O, w, h)
    return O


def default_hyper() -> Hyper:
    hp = Hyper()
    lib().vo_default_hyper(C.byref(hp))
    return hp


def stab_pass(orig3, proc3, flow_fwd, flow_bwd, last_stab, hp: Hyper | None = None, occlusion_mask: bool = False,
              solver_form: str = "exact"):
    """One stabilization pass over frames (t-1, t, t+1); returns (float HWC3, RGBA8).
    occlusion_mask applies the opt-in forward-backward consistency mask;
    solver_form 'fma' solves with the FMA form."""
    hp = hp or default_hyper()
    orig3 = [_c(a, np.float32) for a in orig3]
    proc3 = [_c(a, np.float32) for a in proc3]
    h, w = orig3[0].shape[:2]
    ff = _c(flow_fwd, np.float32)
    fb = _c(flow_bwd, np.float32)
    ls = _c(last_stab, np.float32)
    po = (C.c_void_p * 3)(*[a.ctypes.data for a in orig3])
    pp = (C.c_void_p * 3)(*[a.ctypes.data for a in proc3])
    out = np.empty((h, w, 3), np.float32)
    rgba = np.empty((h, w, 4), np.uint8)
    rc = lib().vo_stab_pass_form(w, h, po, pp, ff, fb, ff.shape[2], ls, C.byref(hp), int(bool(occlusion_mask)),
                                 int(solver_form == "fma"), out, rgba.ctypes.data)
    if rc != 0:
        raise ValueError("vo_stab_pass: invalid sizes")
    return out, rgba


# ---- flow estimator -----------------------------------------------------------

def flow_level_dims(w: int, h: int, level: int):
    a, b, c = _i(), _i(), _i()
    lib().vo_flow_level_dims(w, h, level, C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def flow_weights(level: int):
    lc = (32, 64, 96, 128, 196)[level]
    out = np.empty((lc, 27), np.float32)
    lib().vo_flow_weights(level, out)
    return out


def flow_features(img):
    img = _c(img, np.float32)
    h, w = img.shape[:2]
    out = np.empty(lib().vo_flow_feature_floats(w, h), np.float32)
    lib().vo_flow_features(img, w, h, out)
    return out


def flow_from_features(fa, fb, w: int, h: int):
    out = np.empty((h, w, 3), np.float32)
    lib().vo_flow_from_features(_c(fa, np.float32), _c(fb, np.float32), w, h, out)
    return out


def flow_estimate(img_a, img_b):
    a = _c(img_a, np.float32)
    h, w = a.shape[:2]
    out = np.empty((h, w, 3), np.float32)
    lib().vo_flow_estimate(a, _c(img_b, np.float32), w, h, out)
    return out
