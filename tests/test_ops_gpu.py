"""Correlation and Warp kernels on the GPU, called through the C ABI, against
the CPU restatement and the reference's own CPU ops (golden fixtures).

Tolerances: Correlation is bit-exact (channel-order sum with separately
rounded products, as correlation.cc computes).  Warp is bit-exact against the
single-precision restatement and within 2^-21 * max|input| of the reference's
double-weight CPU op.  The double-precision entry points are bit-exact to the
reference's DOUBLE outputs."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RNG = np.random.Generator(np.random.PCG64(1234))


def _t(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


CORR_SHAPES = [
    ((1, 32, 24, 40), 4), ((2, 7, 13, 17), 4), ((1, 196, 17, 30), 4), ((3, 3, 1, 1), 4), ((1, 16, 5, 33), 3),
    ((1, 9, 11, 12), 2), ((1, 4, 9, 11), 1), ((1, 5, 8, 8), 0), ((1, 6, 20, 21), 6), ((1, 130, 37, 64), 4),
]


@pytest.mark.parametrize("shape,md", CORR_SHAPES)
def test_correlation_bit_exact(vsc, oracle, cuda, shape, md):
    f1 = RNG.standard_normal(shape).astype(np.float32)
    f2 = RNG.standard_normal(shape).astype(np.float32)
    out = vsc.correlation(_t(f1, cuda), _t(f2, cuda), md).cpu().numpy()
    assert np.array_equal(out, oracle.correlation(f1, f2, md))


@pytest.mark.parametrize("shape,md", [((1, 32, 24, 40), 4), ((2, 5, 7, 9), 4), ((1, 3, 6, 6), 2)])
def test_correlation_legacy(vsc, oracle, cuda, shape, md):
    f1 = RNG.standard_normal(shape).astype(np.float32)
    f2 = RNG.standard_normal(shape).astype(np.float32)
    out = vsc.correlation(_t(f1, cuda), _t(f2, cuda), md, legacy=1).cpu().numpy()
    P = 2 * md + 1
    assert out.shape == (shape[0], P * P, shape[2], shape[3])
    assert np.array_equal(out, oracle.correlation(f1, f2, md, legacy=1))


@pytest.mark.parametrize("i", range(5))
def test_correlation_reference_fixture(vsc, cuda, golden, i):
    g = golden["ref_ops"]
    out = vsc.correlation(_t(g[f"corr{i}_f1"], cuda), _t(g[f"corr{i}_f2"], cuda), int(g[f"corr{i}_md"]))
    assert np.array_equal(out.cpu().numpy(), g[f"corr{i}_out"])


def test_correlation_pwc_pyramid_640x360(vsc, oracle, cuda):
    """The Correlation workload of a 640x360 frame pair: the five PWC levels."""
    from vsc_gb300 import synth

    for f1, f2 in synth.feature_pyramid(640, 360, seed=5):
        out = vsc.correlation(_t(f1, cuda), _t(f2, cuda), 4).cpu().numpy()
        assert np.array_equal(out, oracle.correlation(f1, f2, 4))


def test_correlation_full_size_properties(vsc, cuda):
    """1080p level-2 map (480x272, 32 ch): symmetry of the cost volume,
    corr(f1, f2)[d](x) = corr(f2, f1)[-d](x + d), and determinism."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(3)
    f1 = torch.randn((1, 32, 272, 480), device=cuda, generator=g)
    f2 = torch.randn((1, 32, 272, 480), device=cuda, generator=g)
    a = vsc.correlation(f1, f2, 4)
    b = vsc.correlation(f2, f1, 4)
    assert torch.equal(a, vsc.correlation(f1, f2, 4))
    for (dy, dx) in [(1, 3), (-4, 2), (0, -1)]:
        lhs = a[0, dy + 4, dx + 4, max(0, -dy):272 - max(0, dy), max(0, -dx):480 - max(0, dx)]
        rhs = b[0, -dy + 4, -dx + 4, max(0, dy):272 - max(0, -dy), max(0, dx):480 - max(0, -dx)]
        assert torch.allclose(lhs, rhs, rtol=0, atol=1e-4)
    # out-of-map displacements are exactly zero
    assert torch.count_nonzero(a[0, 0, :, :4, :]) == 0


WARP_CASES = [((2, 64, 64, 32), 1.0, 0.0), ((1, 5, 17, 23), 6.0, 3.0), ((1, 3, 4, 4), 10.0, 5.0),
              ((1, 2, 1, 7), 2.0, 1.0), ((3, 11, 30, 29), 20.0, 10.0), ((1, 196, 17, 30), 3.0, 1.5)]


@pytest.mark.parametrize("shape,scale,offset", WARP_CASES)
def test_warp(vsc, oracle, cuda, shape, scale, offset):
    x = (RNG.random(shape) * 10).astype(np.float32)
    flow = (RNG.random((shape[0], 2) + shape[2:]) * scale - offset).astype(np.float32)
    out = vsc.warp(_t(x, cuda), _t(flow, cuda)).cpu().numpy()
    assert np.array_equal(out, oracle.warp_op(x, flow, "f32"))
    ref = oracle.warp_op(x, flow, "refsem")
    assert np.max(np.abs(out - ref)) <= 2.0 ** -21 * np.max(np.abs(x))


@pytest.mark.parametrize("shape", [(2, 3, 37, 70), (1, 8, 33, 65), (1, 16, 9, 130), (3, 5, 12, 64)])
def test_warp_signed_inputs_and_nonfinite_flows(vsc, oracle, cuda, shape):
    """Negative inputs (signed zeros and cancellation in the blend) and flows
    with NaN and infinite entries (no sample taken: 0), for the image-shaped
    3-channel kernel (two pixels per thread, an odd number of rows) and the
    8-channel groups (full and partial)."""
    x = (RNG.random(shape) * 10 - 5).astype(np.float32)
    x.flat[::7] = 0.0
    x.flat[3::11] = -0.0
    flow = (RNG.random((shape[0], 2) + shape[2:]) * 8 - 4).astype(np.float32)
    flow.flat[::13] = np.nan
    flow.flat[5::17] = np.inf
    flow.flat[9::19] = -np.inf
    out = vsc.warp(_t(x, cuda), _t(flow, cuda)).cpu().numpy()
    ref = oracle.warp_op(x, flow, "f32")
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("i", range(3))
def test_warp_reference_fixture(vsc, cuda, golden, i):
    g = golden["ref_ops"]
    x = g[f"warp{i}_x"]
    out = vsc.warp(_t(x, cuda), _t(g[f"warp{i}_flow"], cuda)).cpu().numpy()
    assert np.max(np.abs(out - g[f"warp{i}_out"])) <= 2.0 ** -21 * np.max(np.abs(x))


@pytest.mark.parametrize("i", range(5))
def test_correlation_f64_reference_fixture(vsc, cuda, golden, i):
    """The DOUBLE branch of correlation.cc: bit-exact to the reference's output."""
    g = golden["ref_ops"]
    f1 = g[f"corr{i}_f1"].astype(np.float64)
    f2 = g[f"corr{i}_f2"].astype(np.float64)
    out = vsc.correlation(_t(f1, cuda), _t(f2, cuda), int(g[f"corr{i}_md"]))
    assert np.array_equal(out.cpu().numpy(), g[f"corr{i}_out64"])


@pytest.mark.parametrize("i", range(3))
def test_warp_f64_reference_fixture(vsc, cuda, golden, i):
    """The DOUBLE branch of warp.cc: bit-exact to the reference's output."""
    g = golden["ref_ops"]
    x = g[f"warp{i}_x"].astype(np.float64)
    fl = g[f"warp{i}_flow"].astype(np.float64)
    out = vsc.warp(_t(x, cuda), _t(fl, cuda)).cpu().numpy()
    assert np.array_equal(out, g[f"warp{i}_out64"])


@pytest.mark.parametrize("shape,md", [((2, 37, 19, 45), 4), ((1, 196, 17, 30), 4), ((1, 5, 8, 8), 0)])
def test_ops_f64_vs_restatement(vsc, oracle, cuda, shape, md):
    f1 = RNG.standard_normal(shape)
    f2 = RNG.standard_normal(shape)
    out = vsc.correlation(_t(f1, cuda), _t(f2, cuda), md).cpu().numpy()
    assert out.dtype == np.float64 and np.array_equal(out, oracle.correlation(f1, f2, md))
    fl = RNG.normal(0, 4, (shape[0], 2) + shape[2:])
    fl[0, 0, 0, :3] = [np.nan, 1e9, -0.0]
    w = vsc.warp(_t(f1, cuda), _t(fl, cuda)).cpu().numpy()
    assert np.array_equal(w, oracle.warp_op(f1, fl, "f64"), equal_nan=True)
    with pytest.raises(ValueError, match="legacy"):
        vsc.correlation(_t(f1, cuda), _t(f2, cuda), md, legacy=1)


def test_ops_on_a_side_stream(vsc, oracle, cuda):
    import torch

    s = torch.cuda.Stream()
    f1 = RNG.standard_normal((1, 8, 16, 16)).astype(np.float32)
    with torch.cuda.stream(s):
        a = _t(f1, cuda)
        out = vsc.correlation(a, a, 4, stream=s)
    s.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.correlation(f1, f1, 4))


def test_error_leaves_context_usable(vsc, oracle, cuda):
    import torch

    x = torch.zeros((1, 2, 4, 4), device=cuda)
    with pytest.raises(vsc.VscError):
        vsc.correlation(x, x, 40)
    f = RNG.standard_normal((1, 3, 5, 5)).astype(np.float32)
    assert np.array_equal(vsc.correlation(_t(f, cuda), _t(f, cuda), 4).cpu().numpy(), oracle.correlation(f, f, 4))
