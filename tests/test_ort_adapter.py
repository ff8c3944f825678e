"""The ONNX Runtime adapter (csrc/ort/vsc_ort_ops.cpp), built against the
stand-in ORT headers and runtime of oracle/ort_stub: registration matches the
reference's op library (custom_ops.cpp:18-98), node attributes are read as
correlation.h:19-31 reads them, and Compute on the GPU equals the C ABI."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
STUB = ROOT / "oracle" / "ort_stub"


@pytest.fixture(scope="session")
def ort_lib(vsc, tmp_path_factory):
    import importlib.util

    spec = importlib.util.spec_from_file_location("_b", ROOT / "video-stream-consistency_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    out = tmp_path_factory.mktemp("ort") / "libvsc_ort_stubtest.so"
    b.build_ort(STUB, out, extra_sources=[STUB / "ort_stub_runtime.cc"])
    L = C.CDLL(str(out))
    L.stub_register.argtypes = [C.c_int]
    L.stub_last_error.restype = C.c_char_p
    L.stub_domain_name.restype = C.c_char_p
    cp = C.POINTER(C.c_char_p)
    ip = C.POINTER(C.c_int)
    L.stub_op_info.argtypes = [C.c_int, cp, cp, ip, ip, ip, ip]
    L.stub_set_tensor_type.argtypes = [C.c_int]
    L.stub_run.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_int64), C.c_void_p,
                           C.POINTER(C.c_int64), C.c_void_p, C.POINTER(C.c_int64), C.c_void_p, C.c_size_t,
                           C.POINTER(C.c_int64), ip, C.c_void_p]
    return L


def ops(L):
    out = []
    i = 0
    while True:
        n, p = C.c_char_p(), C.c_char_p()
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        if L.stub_op_info(i, C.byref(n), C.byref(p), C.byref(a), C.byref(b), C.byref(c), C.byref(d)) != 0:
            return out
        out.append((n.value.decode(), p.value.decode(), a.value, b.value, c.value, d.value))
        i += 1


def test_registration_matches_reference(ort_lib):
    assert ort_lib.stub_register(1) == 4
    assert ort_lib.stub_domain_name() == b"custom"
    assert ops(ort_lib) == [("Correlation", "CUDAExecutionProvider", 2, 1, 1, 1),
                            ("Warp", "CUDAExecutionProvider", 2, 1, 1, 1),
                            ("Correlation", "CPUExecutionProvider", 2, 1, 1, 1),
                            ("Warp", "CPUExecutionProvider", 2, 1, 1, 1)]
    # without the CUDA provider only the CPU-provider ops are added (custom_ops.cpp:20-39)
    assert ort_lib.stub_register(0) == 2
    assert [o[1] for o in ops(ort_lib)] == ["CPUExecutionProvider"] * 2


def _run(L, idx, attrs, a, sa, b, sb, out, stream=None):
    names = (C.c_char_p * max(1, len(attrs)))(*[k.encode() for k in attrs])
    vals = (C.c_int64 * max(1, len(attrs)))(*attrs.values())
    oshape = (C.c_int64 * 8)()
    orank = C.c_int()
    rc = L.stub_run(idx, len(attrs), names, vals, a, (C.c_int64 * 4)(*sa), b, (C.c_int64 * 4)(*sb), out[0], out[1],
                    oshape, C.byref(orank), stream)
    return rc, tuple(oshape[: orank.value])


def test_missing_attribute_is_reported(ort_lib):
    ort_lib.stub_register(1)
    buf = (C.c_float * 64)()
    rc, _ = _run(ort_lib, 0, {"max_displacement": 4}, C.addressof(buf), (1, 1, 2, 2), C.addressof(buf),
                 (1, 1, 2, 2), (C.addressof(buf), 256))
    assert rc == -1 and b"legacy" in ort_lib.stub_last_error()


@pytest.mark.gpu
def test_compute_cuda_and_cpu_providers(ort_lib, vsc, oracle, cuda):
    import torch

    ort_lib.stub_register(1)
    rng = np.random.Generator(np.random.PCG64(5))
    f1 = rng.standard_normal((2, 8, 12, 20)).astype(np.float32)
    f2 = rng.standard_normal((2, 8, 12, 20)).astype(np.float32)
    ref = oracle.correlation(f1, f2, 4)
    # CUDA provider: device tensors on the context's stream
    d1, d2 = torch.from_numpy(f1).to(cuda), torch.from_numpy(f2).to(cuda)
    dout = torch.empty(ref.shape, dtype=torch.float32, device=cuda)
    s = torch.cuda.current_stream()
    rc, shp = _run(ort_lib, 0, {"legacy": 0, "max_displacement": 4}, d1.data_ptr(), f1.shape, d2.data_ptr(),
                   f2.shape, (dout.data_ptr(), dout.numel() * 4), C.c_void_p(s.cuda_stream))
    assert rc == 0, ort_lib.stub_last_error()
    assert shp == (2, 9, 9, 12, 20)
    assert np.array_equal(dout.cpu().numpy(), ref)
    # CPU provider: host tensors, staged through the device
    hout = np.empty(ref.shape, np.float32)
    rc, shp = _run(ort_lib, 2, {"legacy": 0, "max_displacement": 4}, f1.ctypes.data, f1.shape, f2.ctypes.data,
                   f2.shape, (hout.ctypes.data, hout.nbytes))
    assert rc == 0, ort_lib.stub_last_error()
    assert np.array_equal(hout, ref)
    # legacy on the CPU provider is refused, as correlation.h:45-46 does
    rc, _ = _run(ort_lib, 2, {"legacy": 1, "max_displacement": 4}, f1.ctypes.data, f1.shape, f2.ctypes.data,
                 f2.shape, (hout.ctypes.data, hout.nbytes))
    assert rc == -1 and b"Legacy" in ort_lib.stub_last_error()
    # Warp on both providers
    x = (rng.random((1, 5, 9, 11)) * 10).astype(np.float32)
    fl = (rng.random((1, 2, 9, 11)) * 4 - 2).astype(np.float32)
    wref = oracle.warp_op(x, fl, "f32")
    wout = np.empty_like(x)
    rc, shp = _run(ort_lib, 3, {}, x.ctypes.data, x.shape, fl.ctypes.data, fl.shape, (wout.ctypes.data, wout.nbytes))
    assert rc == 0 and shp == x.shape and np.array_equal(wout, wref)
    dx, dfl = torch.from_numpy(x).to(cuda), torch.from_numpy(fl).to(cuda)
    dw = torch.empty_like(dx)
    rc, _ = _run(ort_lib, 1, {}, dx.data_ptr(), x.shape, dfl.data_ptr(), fl.shape, (dw.data_ptr(), dw.numel() * 4),
                 C.c_void_p(s.cuda_stream))
    assert rc == 0 and np.array_equal(dw.cpu().numpy(), wref)


@pytest.mark.gpu
def test_double_tensors(ort_lib, vsc, cuda, golden):
    """DOUBLE inputs: the CPU provider computes them as correlation.cc / warp.cc
    do (bit-exact to the reference's double outputs); the CUDA provider
    accepts FLOAT only, like the reference's CUDA kernels."""
    g = golden["ref_ops"]
    ort_lib.stub_register(1)
    ort_lib.stub_set_tensor_type(11)  # ONNX_TENSOR_ELEMENT_DATA_TYPE_DOUBLE
    try:
        f1 = g["corr0_f1"].astype(np.float64)
        f2 = g["corr0_f2"].astype(np.float64)
        ref = g["corr0_out64"]
        hout = np.empty(ref.shape, np.float64)
        rc, shp = _run(ort_lib, 2, {"legacy": 0, "max_displacement": int(g["corr0_md"])}, f1.ctypes.data, f1.shape,
                       f2.ctypes.data, f2.shape, (hout.ctypes.data, hout.nbytes))
        assert rc == 0, ort_lib.stub_last_error()
        assert np.array_equal(hout, ref)
        x = g["warp0_x"].astype(np.float64)
        fl = g["warp0_flow"].astype(np.float64)
        wout = np.empty_like(x)
        rc, _ = _run(ort_lib, 3, {}, x.ctypes.data, x.shape, fl.ctypes.data, fl.shape, (wout.ctypes.data, wout.nbytes))
        assert rc == 0 and np.array_equal(wout, g["warp0_out64"])
        # the CUDA provider refuses doubles
        import torch

        s = torch.cuda.current_stream()
        d1 = torch.from_numpy(f1).to(cuda)
        dout = torch.empty(ref.shape, dtype=torch.float64, device=cuda)
        rc, _ = _run(ort_lib, 0, {"legacy": 0, "max_displacement": 4}, d1.data_ptr(), f1.shape, d1.data_ptr(),
                     f1.shape, (dout.data_ptr(), dout.numel() * 8), C.c_void_p(s.cuda_stream))
        assert rc == -1 and b"float" in ort_lib.stub_last_error()
    finally:
        ort_lib.stub_set_tensor_type(1)  # FLOAT
