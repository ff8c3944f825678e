"""Reduced-precision Correlation on the tensor cores (tcgen05, BF16 / FP16
operands, FP32 accumulation) through the C ABI, against the FP64 restatement
of correlation.cc (which equals the reference's own double-precision op).

Bars, per output element with S = sum_c f1 f2 and A = sum_c |f1 f2|:
  |out - S| <= (2u + u^2 + C 2^-22) A + 1e-6,  u = 2^-8 (BF16), 2^-11 (FP16)
(operand rounding, then FP32 accumulation).  Features whose values are
exact in 16 bits give sums exact in FP32: those must match bit for bit,
which pins the tile indexing independently of rounding."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RNG = np.random.Generator(np.random.PCG64(99))
U = {"bf16": 2.0 ** -8, "fp16": 2.0 ** -11}


def _t(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _bound_check(out, f1, f2, md, dtype, oracle):
    exact = oracle.correlation(f1.astype(np.float64), f2.astype(np.float64), md)
    absd = oracle.correlation(np.abs(f1).astype(np.float64), np.abs(f2).astype(np.float64), md)
    u = U[dtype]
    C = f1.shape[1]
    err = np.abs(out.astype(np.float64) - exact)
    bound = (2 * u + u * u + C * 2.0 ** -22) * absd + 1e-6
    assert np.all(err <= bound), float(np.max(err / bound))
    return float(err.max()), float(np.sqrt(np.mean(err ** 2)))


SHAPES = [((1, 32, 24, 40), 4), ((2, 7, 13, 17), 4), ((1, 196, 17, 30), 4), ((1, 64, 9, 300), 4),
          ((1, 130, 5, 129), 3), ((1, 1, 4, 4), 1), ((2, 16, 6, 128), 0), ((1, 24, 20, 150), 8)]


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,md", SHAPES)
def test_lowp_correlation_error_bound(vsc, oracle, cuda, shape, md, dtype):
    f1 = RNG.standard_normal(shape).astype(np.float32)
    f2 = RNG.standard_normal(shape).astype(np.float32)
    out = vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), md, dtype).cpu().numpy()
    P = 2 * md + 1
    assert out.shape == (shape[0], P, P, shape[2], shape[3])
    _bound_check(out, f1, f2, md, dtype, oracle)
    vsc.check_device()


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
@pytest.mark.parametrize("shape,md", [((1, 32, 24, 40), 4), ((2, 48, 7, 260), 4), ((1, 200, 5, 33), 2)])
def test_lowp_correlation_exact_on_representable_values(vsc, oracle, cuda, shape, md, dtype):
    """Small integers times a power of two are exact in BF16 and FP16 and so
    are their products and (short) sums in FP32: the result must be the
    reference sum bit for bit, whatever the per-level scale."""
    f1 = (RNG.integers(-3, 4, shape) * 0.25).astype(np.float32)
    f2 = (RNG.integers(-3, 4, shape) * 0.5).astype(np.float32)
    out = vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), md, dtype).cpu().numpy()
    assert np.array_equal(out, oracle.correlation(f1, f2, md))
    vsc.check_device()


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
def test_lowp_correlation_pwc_pyramid_640x360(vsc, oracle, cuda, dtype):
    """The five PWC levels of a 640x360 frame pair (C = 32..196); error
    statistics against FP64 for the record."""
    from vsc_gb300 import synth

    stats = []
    for f1, f2 in synth.feature_pyramid(640, 360, seed=5):
        out = vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), 4, dtype).cpu().numpy()
        stats.append(_bound_check(out, f1, f2, 4, dtype, oracle))
    print(dtype, "max-abs / rms error per level:", stats)
    vsc.check_device()


def test_lowp_correlation_caller_workspace_and_errors(vsc, oracle, cuda):
    import torch

    f1 = RNG.standard_normal((1, 16, 10, 20)).astype(np.float32)
    f2 = RNG.standard_normal((1, 16, 10, 20)).astype(np.float32)
    need = vsc.load().vsc_correlation_lowp_workspace_size(1, 16, 10, 20)
    ws = torch.empty(need, dtype=torch.uint8, device=cuda)
    a = vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), 4, "bf16", workspace=ws).cpu().numpy()
    b = vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), 4, "bf16").cpu().numpy()
    assert np.array_equal(a, b)
    with pytest.raises(vsc.VscError, match="ENOMEM"):
        vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), 4, "bf16", workspace=ws[: need // 2])
    big = torch.zeros((1, 209, 4, 4), device=cuda)
    with pytest.raises(vsc.VscError, match="EUNSUPPORTED"):
        vsc.correlation_lowp(big, big, 4, "bf16")
    with pytest.raises(vsc.VscError, match="EUNSUPPORTED"):
        vsc.correlation_lowp(_t(f1, cuda), _t(f2, cuda), 9, "bf16")
    vsc.check_device()


def _psnr(a, b):
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(1.0 / mse)


@pytest.mark.parametrize("dtype", ["bf16", "fp16"])
def test_stabilizer_tensor_core_flow_vs_plain(vsc, cuda, dtype):
    """The precision form of the whole step: the flow estimator's correlations
    on the tensor cores, everything else FP32.  Bar: stabilized output within
    40 dB PSNR of the plain method's, frame after frame."""
    from vsc_gb300 import synth

    w, h = 256, 144
    s = synth.SyntheticStream(w, h, seed=17)
    frames = [s.frame(i) for i in range(8)]
    plain = vsc.Stabilizer(w, h)
    low = vsc.Stabilizer(w, h, corr_dtype=dtype)
    for st in (plain, low):
        for i in range(3):
            st.load_frame(*frames[i])
    worst = float("inf")
    for t in range(1, 6):
        plain.step()
        low.step()
        a, b = plain.buffer(0).cpu().numpy(), low.buffer(0).cpu().numpy()
        worst = min(worst, _psnr(a, b))
        fa, fb = plain.buffer(1).cpu().numpy(), low.buffer(1).cpu().numpy()
        assert np.mean(np.abs(fa - fb)) < 0.25  # flows mostly agree (pixels)
        for st in (plain, low):
            st.load_frame(*frames[t + 2])
    plain.close()
    low.close()
    assert worst >= 40.0, worst
    vsc.check_device()
