"""The C ABI without a GPU: libvsc.so loads, exports exactly what
include/vsc.h declares, and rejects invalid arguments before touching the
device (status codes, never exit())."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "vsc.h").read_text()
    return sorted(set(re.findall(r"VSC_API\s+[\w\s\*]+?\b(vsc_\w+)\s*\(", text)))


def test_header_and_python_list_agree(vsc):
    assert declared_symbols() == sorted(vsc.EXPORTED)


def test_library_exports_every_declared_symbol(vsc):
    lib = vsc.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(vsc.LIB_PATH)], capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r"\bT (vsc_\w+)", out)))
    assert exported == declared_symbols()


def test_built_for_sm103a_only():
    import importlib.util

    spec = importlib.util.spec_from_file_location("_b", ROOT / "video-stream-consistency_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-fmad=false" in mod.COMMON


def test_version_and_defaults(vsc):
    assert vsc.load().vsc_version() >= 100
    hp = vsc.default_hyper_params()
    assert (hp.alpha, hp.beta, hp.gamma, hp.pyramid_levels, hp.num_iter) == (6800.0, 6800.0, 2.0, 2, 150)
    assert abs(hp.step_size - 0.15) < 1e-7 and abs(hp.mom_fac - 0.15) < 1e-7
    assert vsc.consist_out_workspace_size(1920, 1080) == 1920 * 1080 * 12 * 4
    assert vsc.consist_out_workspace_size(0, 10) == 0


def _status(vsc, rc):
    return rc, vsc.load().vsc_last_error().decode()


def test_ops_reject_bad_arguments(vsc):
    L = vsc.load()
    p = C.c_void_p(16)
    rc, msg = _status(vsc, L.vsc_correlation_fwd(None, p, p, 1, 1, 4, 4, 4, 0, None))
    assert rc == vsc.VSC_EINVAL and "null" in msg
    rc, msg = _status(vsc, L.vsc_correlation_fwd(p, p, p, 1, 0, 4, 4, 4, 0, None))
    assert rc == vsc.VSC_EINVAL and "shape" in msg
    rc, msg = _status(vsc, L.vsc_correlation_fwd(p, p, p, 1, 1, 4, 4, 40, 0, None))
    assert rc == vsc.VSC_EINVAL and "max_displacement" in msg
    rc, msg = _status(vsc, L.vsc_correlation_fwd(p, p, p, 1, 1, 4, 4, 4, 2, None))
    assert rc == vsc.VSC_EINVAL and "legacy" in msg
    rc, msg = _status(vsc, L.vsc_warp_fwd(p, None, p, 1, 1, 4, 4, None))
    assert rc == vsc.VSC_EINVAL
    rc, msg = _status(vsc, L.vsc_warp_fwd(p, p, p, -1, 1, 4, 4, None))
    assert rc == vsc.VSC_EINVAL


def test_stabilization_kernels_reject_bad_images(vsc):
    L = vsc.load()
    good = vsc.Image(16, 8, 8, 3)
    other = vsc.Image(16, 9, 8, 3)
    two = vsc.Image(16, 8, 8, 2)
    null = vsc.Image(None, 8, 8, 3)
    rc, msg = _status(vsc, L.vsc_get_warp_result(C.byref(good), C.byref(good), C.byref(other), None))
    assert rc == vsc.VSC_EINVAL and "size" in msg
    rc, msg = _status(vsc, L.vsc_get_warp_result(C.byref(two), C.byref(good), C.byref(good), None))
    assert rc == vsc.VSC_EINVAL and "channels" in msg
    rc, msg = _status(vsc, L.vsc_get_consist_wt(C.byref(good), C.byref(null), C.byref(good), 1.0, 1.0, None))
    assert rc == vsc.VSC_EINVAL and "null" in msg
    rc, msg = _status(vsc, L.vsc_get_bilinear(C.byref(good), C.byref(two), None))
    assert rc == vsc.VSC_EINVAL and "channel" in msg
    rc, msg = _status(vsc, L.vsc_get_consist_out(C.byref(good), C.byref(good), C.byref(good), -1, 0.1, 0.1,
                                                 C.byref(good), None, 0, None))
    assert rc == vsc.VSC_EINVAL and "negative" in msg
    rc, msg = _status(vsc, L.vsc_get_consist_out(C.byref(good), C.byref(good), C.byref(good), 3, 0.1, 0.1,
                                                 C.byref(good), C.c_void_p(16), 10, None))
    assert rc == vsc.VSC_ENOMEM and "workspace" in msg
    rc, msg = _status(vsc, L.vsc_char_to_float_image(C.c_void_p(17), C.byref(good), None))
    assert rc == vsc.VSC_EINVAL and "aligned" in msg


def test_stabilizer_rejects_bad_config(vsc):
    L = vsc.load()
    h = C.c_void_p()
    for cfg, code, word in [
        (vsc.StabilizerConfig(4, 4, 1, 1, 1, 3, 1), vsc.VSC_EINVAL, "size"),
        (vsc.StabilizerConfig(64, 64, 2, 1, 1, 3, 1), vsc.VSC_EUNSUPPORTED, "batch"),
        (vsc.StabilizerConfig(64, 64, 1, 1, 0, 3, 1), vsc.VSC_EINVAL, "downscale"),
        (vsc.StabilizerConfig(64, 64, 1, 0, 1, 4, 1), vsc.VSC_EINVAL, "flow_channels"),
        (vsc.StabilizerConfig(64, 64, 1, 1, 1, 3, 1, 7), vsc.VSC_EINVAL, "corr_dtype"),
    ]:
        rc, msg = _status(vsc, L.vsc_stabilizer_create(C.byref(cfg), None, C.byref(h)))
        assert rc == code and word in msg, (rc, msg)
    rc, _ = _status(vsc, L.vsc_stabilizer_create(None, None, C.byref(h)))
    assert rc == vsc.VSC_EINVAL
    rc, _ = _status(vsc, L.vsc_stabilizer_step(None, None, 0))
    assert rc == vsc.VSC_EINVAL
    assert L.vsc_stabilizer_destroy(None) == vsc.VSC_OK
    assert L.vsc_stabilizer_last_launches(None) == 0
    assert not L.vsc_stabilizer_hyper_params(None)


def test_product_never_touches_the_oracle():
    """No product file names the checker's library or module."""
    pkg = ROOT / "video-stream-consistency_gb300"
    for f in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cpp")) + list(pkg.rglob("*.h")):
        text = f.read_text()
        assert "liboracle" not in text and "import oracle" not in text and "vsc_oracle" not in text, f
