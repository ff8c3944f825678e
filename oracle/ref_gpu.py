"""ctypes front end of the reference-GPU harness (test infrastructure only).

Runs the reference's own CUDA kernels — compiled in place from the reference
tree into oracle/_ref/ref_kernels_{exact,default}.cubin — through
oracle/_build/librefgpu.so, with the reference's launch geometry and call
sequence (see ref_gpu/ref_gpu_harness.cu).  Tensors are torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "librefgpu.so"
CUBINS = {"exact": HERE / "_ref" / "ref_kernels_exact.cubin", "default": HERE / "_ref" / "ref_kernels_default.cubin"}


class Img(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("channels", C.c_int)]


# entry points of ref_gpu/ref_gpu_harness.cu (besides rg_last_error)
FUNCS = ("rg_init", "rg_warp", "rg_adap_comb", "rg_consist_wt", "rg_bilinear", "rg_consist_out", "rg_to_float",
         "rg_to_char", "rg_correlation", "rg_correlation_legacy", "rg_warp_op", "rg_stab_pass")

_libs: dict = {}


def available(kind: str = "exact") -> bool:
    return LIB.exists() and CUBINS[kind].exists()


def load(kind: str = "exact"):
    """One library instance per cubin kind (each holds its own module)."""
    if kind in _libs:
        return _libs[kind]
    import shutil
    import tempfile

    # a private copy of the library per kind, so each keeps its own module
    tmp = Path(tempfile.mkdtemp()) / f"librefgpu_{kind}.so"
    shutil.copy(LIB, tmp)
    L = C.CDLL(str(tmp))
    L.rg_last_error.restype = C.c_char_p
    for fn in FUNCS:
        getattr(L, fn).restype = C.c_int
    L.rg_init.argtypes = [C.c_char_p]
    L.rg_warp.argtypes = [Img, Img, Img]
    L.rg_adap_comb.argtypes = [Img] * 9 + [C.c_float]
    L.rg_consist_wt.argtypes = [Img, Img, Img, C.c_float, C.c_float]
    L.rg_bilinear.argtypes = [Img, Img]
    L.rg_consist_out.argtypes = [Img, Img, Img, C.c_int, C.c_float, C.c_float, Img]
    L.rg_to_float.argtypes = [C.c_void_p, Img]
    L.rg_to_char.argtypes = [Img, C.c_void_p]
    L.rg_correlation.argtypes = [C.c_void_p] * 3 + [C.c_int] * 5 + [C.c_void_p]
    L.rg_correlation_legacy.argtypes = [C.c_void_p] * 3 + [C.c_int] * 5 + [C.c_void_p]
    L.rg_warp_op.argtypes = [C.c_void_p] * 3 + [C.c_int] * 4 + [C.c_void_p]
    L.rg_stab_pass.argtypes = [C.POINTER(Img), C.POINTER(Img), C.POINTER(Img), C.POINTER(Img), C.c_int, C.c_int,
                               C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p]
    if L.rg_init(str(CUBINS[kind]).encode()) != 0:
        raise RuntimeError(L.rg_last_error().decode())
    _libs[kind] = L
    return L


def img(t) -> Img:
    h, w, c = t.shape
    return Img(t.data_ptr(), w, h, c)


def check(L, rc):
    if rc != 0:
        raise RuntimeError(L.rg_last_error().decode())
