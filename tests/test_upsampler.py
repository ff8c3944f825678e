"""Learned flow upsampler (vsc_upsampler_*): the tensor-core inference (FP16
weights and activations, FP32 accumulation) against a float64 numpy
restatement of the net that rounds the same operands to FP16, and against
the same net in FP32 (the error FP16 costs); the bilinear fallback; training
that overfits a small batch; the stabilizer's fast mode with the net
attached, whose two flows (one batched launch) equal single-image calls."""
from __future__ import annotations

import numpy as np
import pytest

RNG = np.random.Generator(np.random.PCG64(31))
LAYERS = [(3, 32), (32, 32), (32, 32), (32, 2)]


def test_param_count(vsc):
    n = sum(co * 9 * ci + co for ci, co in LAYERS)
    assert vsc.Upsampler.param_count() == n == 19970


def _np_forward(params, inp, half_acts=False):
    """The net in float64: 3x3 zero-padded convolutions, ReLU between; with
    half_acts the input and every inner activation are rounded to FP16 (the
    tensor-core path's operands)."""
    rnd = (lambda a: a.astype(np.float16).astype(np.float64)) if half_acts else (lambda a: a)  # noqa: E731
    x = rnd(inp.astype(np.float64))
    off = 0
    for li, (ci, co) in enumerate(LAYERS):
        w = params[off:off + co * 9 * ci].reshape(co, 3, 3, ci).astype(np.float64)
        off += co * 9 * ci
        b = params[off:off + co].astype(np.float64)
        off += co
        h, wd = x.shape[:2]
        xp = np.pad(x, ((1, 1), (1, 1), (0, 0)))
        y = np.tile(b, (h, wd, 1))
        for ky in range(3):
            for kx in range(3):
                y += xp[ky:ky + h, kx:kx + wd] @ w[:, ky, kx, :].T
        x = rnd(np.maximum(y, 0)) if li < 3 else y
    return x


def _base(coarse, w, h):
    """Bilinear upsampling (kernel_bilinear's sampling) with vectors scaled."""
    ch, cw = coarse.shape[:2]
    out = np.empty((h, w, 2))
    for y in range(h):
        for x in range(w):
            xx, yy = np.float32(x * cw / w), np.float32(y * ch / h)
            ix, iy = min(int(np.floor(xx)), cw - 1), min(int(np.floor(yy)), ch - 1)
            fx, fy = xx - ix, yy - iy
            ix1, iy1 = min(ix + 1, cw - 1), min(iy + 1, ch - 1)
            v = (coarse[iy, ix, :2] * (1 - fx) * (1 - fy) + coarse[iy, ix1, :2] * fx * (1 - fy)
                 + coarse[iy1, ix, :2] * (1 - fx) * fy + coarse[iy1, ix1, :2] * fx * fy)
            out[y, x] = v * np.array([w / cw, h / ch])
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("h,w", [(24, 36), (45, 261)])
def test_inference_matches_numpy_and_fallback(vsc, cuda, h, w):
    """(45, 261): three 128-pixel segments, the last one partial, and a
    partial band of rows."""
    import torch

    coarse = RNG.normal(0, 1.5, (h // 2, w // 2, 3)).astype(np.float32)
    frame = RNG.random((h, w, 3)).astype(np.float32)
    params = (RNG.normal(0, 0.08, vsc.Upsampler.param_count())).astype(np.float32)
    up = vsc.Upsampler(params)
    dc, df = torch.from_numpy(coarse).to(cuda), torch.from_numpy(frame).to(cuda)
    inp = vsc.Upsampler.prepare(dc, df).cpu().numpy()
    base = _base(coarse, w, h)
    assert np.allclose(inp[..., :2], base, atol=1e-5)
    lum = frame @ np.array([0.299, 0.587, 0.114])
    assert np.allclose(inp[..., 2], lum, atol=1e-6)
    p16 = params.astype(np.float16).astype(np.float32)  # inference weights are FP16
    for i, (ci, co) in enumerate(LAYERS):  # biases stay FP32
        start = sum(c * 9 * a + c for a, c in LAYERS[:i]) + co * 9 * ci
        p16[start:start + co] = params[start:start + co]
    r = _np_forward(p16, inp, half_acts=True)
    up.set_max_residual(1e9)
    got = up.apply(dc, df).cpu().numpy()
    # same FP16 operands, FP32 vs float64 accumulation (an activation's FP16
    # rounding may flip one unit where the two sums straddle a rounding point)
    assert np.allclose(got[..., :2], inp[..., :2] + r, atol=1e-3 * (1 + np.abs(r).max()))
    assert np.all(got[..., 2] == 0)
    # the cost of FP16 activations against the net in FP32 (FP16 weights in both)
    r32 = _np_forward(p16, inp)
    assert np.abs(got[..., :2] - (inp[..., :2] + r32)).max() <= 2e-2 * (1 + np.abs(r32).max())
    up.set_max_residual(0.0)  # every residual is refused: the bilinear base
    got0 = up.apply(dc, df).cpu().numpy()
    keep = np.max(np.abs(r), -1) > 1e-3
    assert np.array_equal(got0[..., :2][keep], inp[..., :2][keep])
    up.close()


@pytest.mark.gpu
def test_training_overfits_a_batch(vsc, cuda):
    import torch

    n, h, w = 4, 32, 32
    inp = torch.from_numpy(RNG.normal(0, 1, (n, h, w, 3)).astype(np.float32)).to(cuda)
    # target: the base shifted by a smooth function of the luma channel
    tgt = (inp[..., :2] + 0.3 * torch.tanh(inp[..., 2:3])).contiguous()
    up = vsc.Upsampler()
    first = up.train_step(inp, tgt, 3e-3)
    for _ in range(400):
        last = up.train_step(inp, tgt, 3e-3)
    assert last < 0.5 * first, (first, last)
    p = up.params()
    assert np.all(np.isfinite(p))
    up.close()


@pytest.mark.gpu
def test_stabilizer_with_learned_upsampler(vsc, cuda):
    """FLOWDOWNSCALE=2 with the net attached: runs, differs from the bilinear
    fast mode, and with every residual refused uses the scaled bilinear base."""
    from vsc_gb300 import synth

    w, h = 128, 96
    s = synth.SyntheticStream(w, h, seed=71)
    frames = [s.frame(i) for i in range(5)]
    a = vsc.Stabilizer(w, h, flow_downscale=2)
    b = vsc.Stabilizer(w, h, flow_downscale=2)
    up = vsc.Upsampler(RNG.normal(0, 0.05, vsc.Upsampler.param_count()).astype(np.float32))
    up.set_max_residual(1e9)
    b.set_upsampler(up)
    for st in (a, b):
        for i in range(3):
            st.load_frame(*frames[i])
        st.step()
    fa, fb = a.buffer(1).cpu().numpy(), b.buffer(1).cpu().numpy()
    assert not np.allclose(fa, fb)
    # both flows come from one batched launch; each equals the single-image call
    # on the same coarse flow and frame (flow(I1 -> I2) with I1, flow(I2 -> I1) with I2)
    import torch

    from vsc_gb300.train_upsampler import nearest

    f1, f2 = (vsc.char_to_float_image(torch.from_numpy(frames[i][0]).to(cuda)) for i in (1, 2))
    ab, ba = vsc.flow_estimate(nearest(f1, w // 2, h // 2), nearest(f2, w // 2, h // 2))
    assert np.allclose(up.apply(ab, f1).cpu().numpy(), fb, atol=1e-5)
    assert np.allclose(up.apply(ba, f2).cpu().numpy(), b.buffer(2).cpu().numpy(), atol=1e-5)
    with pytest.raises(vsc.VscError, match="ESTATE"):
        vsc.Stabilizer(w, h).set_upsampler(up)
    a.close()
    b.close()
    up.close()
