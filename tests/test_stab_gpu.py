"""Stabilization pass on the GPU through the C ABI, against the CPU
restatement of flowconsistency.cu / gpuimage.cu / videostabilizer.cpp.

Tolerance: none — every kernel of the pass (frame I/O, warps, adaptive
combination, consistency weights, pyramid, solver, flow estimator) is
bit-exact to the restatement, so the comparisons are exact equality."""
from __future__ import annotations

import numpy as np
import pytest

from oracle_driver import run_oracle_stream

pytestmark = pytest.mark.gpu
RNG = np.random.Generator(np.random.PCG64(4321))


def _t(a, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _img(h, w, c=3, lo=0.0, hi=1.0):
    return RNG.uniform(lo, hi, (h, w, c)).astype(np.float32)


def test_rgba_round_trip(vsc, oracle, cuda):
    rgba = RNG.integers(0, 256, (37, 53, 4), dtype=np.uint8)
    f = vsc.char_to_float_image(_t(rgba, cuda))
    assert np.array_equal(f.cpu().numpy(), oracle.rgba_to_float(rgba))
    back = vsc.float_to_char_image(f).cpu().numpy()
    assert np.array_equal(back, oracle.float_to_rgba(oracle.rgba_to_float(rgba)))
    special = np.array([1.0, 1.01, -0.5, 2.0, np.nan, 1e30, 0.999, -1.0, 256.0 / 255.0, np.inf, -np.inf, 1e-40],
                       np.float32).reshape(2, 2, 3)
    got = vsc.float_to_char_image(_t(special, cuda)).cpu().numpy()
    assert np.array_equal(got, oracle.float_to_rgba(special))


def test_rgba_unaligned_and_ragged(vsc, oracle, cuda):
    """Pointers off the 16-byte grid and pixel counts not divisible by 4 take
    the one-pixel-per-thread kernels; results are the same bits."""
    import ctypes as C
    import torch

    rgba = RNG.integers(0, 256, (7, 9, 4), dtype=np.uint8)  # 63 pixels
    ref = oracle.rgba_to_float(rgba)
    big = torch.zeros(63 * 4 + 4, dtype=torch.uint8, device=cuda)
    big[4:] = torch.from_numpy(rgba.reshape(-1)).to(cuda)
    outbuf = torch.zeros(63 * 3 + 1, dtype=torch.float32, device=cuda)
    img = vsc.Image(outbuf.data_ptr() + 4, 9, 7, 3)
    vsc._check(vsc.load().vsc_char_to_float_image(C.c_void_p(big.data_ptr() + 4), C.byref(img), None))
    torch.cuda.synchronize()
    assert np.array_equal(outbuf[1:].cpu().numpy().reshape(7, 9, 3), ref)
    back = torch.zeros(63 * 4 + 4, dtype=torch.uint8, device=cuda)
    vsc._check(vsc.load().vsc_float_to_char_image(C.byref(img), C.c_void_p(back.data_ptr() + 4), None))
    torch.cuda.synchronize()
    assert np.array_equal(back[4:].cpu().numpy().reshape(7, 9, 4), oracle.float_to_rgba(ref))


@pytest.mark.parametrize("h,w,fc,scale", [(24, 32, 3, 4.0), (17, 29, 2, 12.0), (5, 4, 3, 50.0), (64, 96, 2, 0.5)])
def test_warp_result(vsc, oracle, cuda, h, w, fc, scale):
    img = _img(h, w)
    flow = RNG.normal(0, scale, (h, w, fc)).astype(np.float32)
    got = vsc.get_warp_result(_t(img, cuda), _t(flow, cuda)).cpu().numpy()
    assert np.array_equal(got, oracle.stab_warp(img, flow))


@pytest.mark.parametrize("alpha,beta,gamma", [(6800.0, 6800.0, 2.0), (20.0, 6800.0, 2.0), (50.0, 900.0, 0.5)])
def test_adap_comb_and_weights(vsc, oracle, cuda, alpha, beta, gamma):
    h, w = 31, 47
    base = _img(h, w)
    ims = [np.clip(base + RNG.normal(0, s, base.shape), 0, 1).astype(np.float32)
           for s in (0.0, 0.08, 0.1, 0.005, 0.12, 0.01, 0.004)]
    ain, apr = vsc.get_adap_comb(*[_t(a, cuda) for a in ims], alpha)
    oin, opr = oracle.adap_comb(*ims, alpha)
    assert np.array_equal(ain.cpu().numpy(), oin)
    assert np.array_equal(apr.cpu().numpy(), opr)
    wt = vsc.get_consist_wt(ain, _t(ims[0], cuda), beta, gamma).cpu().numpy()
    owt = oracle.consist_wt(ims[0], oin, beta, gamma)
    assert np.array_equal(wt, owt)
    if alpha < beta:
        # both branches of the 1e-3 clamp are exercised
        assert (owt == 0).any() and (owt > 0).any()


@pytest.mark.parametrize("src,dst", [((64, 48), (32, 24)), ((33, 21), (16, 10)), ((16, 10), (33, 21)),
                                     ((1920, 1080), (960, 540)), ((960, 540), (1920, 1080)),
                                     # exact 2x (the staged kernel): partial blocks, rows that are
                                     # not 16-byte aligned, one pixel, one block's window edges
                                     ((16, 10), (32, 20)), ((481, 67), (962, 134)), ((1, 1), (2, 2)),
                                     ((65, 5), (130, 10)), ((640, 360), (1280, 720))])
def test_bilinear(vsc, oracle, cuda, src, dst):
    img = _img(src[1], src[0])
    got = vsc.get_bilinear(_t(img, cuda), dst[0], dst[1]).cpu().numpy()
    assert np.array_equal(got, oracle.bilinear(img, dst[0], dst[1]))


def test_bilinear_2x_special_values(vsc, oracle, cuda):
    """The staged exact-2x path propagates Inf and NaN and keeps signed zeros
    exactly as the per-pixel expression does."""
    img = _img(37, 70)
    img[3, 5, 0] = np.inf
    img[10, 20, 1] = -np.inf
    img[20, 33, 2] = np.nan
    img[0, 0, :] = -0.0
    img[-1, -1, :] = np.float32(3.0e38)
    got = vsc.get_bilinear(_t(img, cuda), 140, 74).cpu().numpy()
    ref = oracle.bilinear(img, 140, 74)
    nan = np.isnan(ref)
    assert nan.any() and np.isinf(ref).any()
    assert np.array_equal(np.isnan(got), nan)  # NaN payloads differ between CPU and GPU arithmetic
    assert np.array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))


def _equal_up_to_zero_sign(a, b):
    """Equal as IEEE values, and where the bits differ both are zeros: the
    solver sums a pixel's neighbours from the first term, the oracle (as the
    reference) onto 0.0f, which can change only the sign of a zero."""
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    if not np.array_equal(a, b):
        return False
    differ = a.view(np.uint32) != b.view(np.uint32)
    return bool(np.all(a[differ] == 0))


# widths divisible by 4 take the persistent TMA-fed kernel, others the
# per-tile kernel; iteration counts not divisible by 8 end in a short launch
@pytest.mark.parametrize("h,w,iters", [(9, 11, 0), (9, 11, 1), (9, 11, 2), (40, 56, 75), (3, 3, 5), (2, 2, 4),
                                       (67, 33, 150), (48, 200, 13), (540, 960, 75), (1080, 1920, 9),
                                       (1080, 1920, 150), (17, 4, 3), (100, 64, 150)])
def test_consist_out(vsc, oracle, cuda, h, w, iters):
    import torch

    P, A, Wt, O0 = _img(h, w), _img(h, w), _img(h, w, hi=2.0), _img(h, w)
    O = _t(O0, cuda)
    vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), iters, 0.15, 0.15, O)
    ref = oracle.consist_out(P, A, Wt, iters, 0.15, 0.15, O0)
    assert _equal_up_to_zero_sign(O.cpu().numpy(), ref)
    # caller-provided workspace gives the same bits
    ws = torch.empty(vsc.consist_out_workspace_size(w, h) // 4, dtype=torch.float32, device=cuda)
    O2 = _t(O0, cuda)
    vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), iters, 0.15, 0.15, O2, workspace=ws)
    assert np.array_equal(O2.cpu().numpy().view(np.uint32), O.cpu().numpy().view(np.uint32))


# the FMA form: widths divisible by 4 take the TMA-fed kernel (128 x 72 tiles
# of one plane: these sizes give one tile, several, partial tiles at the right
# and bottom), others the plain-load one; iteration counts not divisible by 8
# end in a short launch.  Border tiles test the frame's rows 0, h - 2 and
# h - 1 and its columns 0, w - 2 and w - 1 at fixed places when the bottom row
# of tiles can be moved to end on the frame's last row, per pixel otherwise:
# 61 rows leave it in place (rows h - 2 and h - 1 in two warps), 72, 100, 120
# and 130 rows move it over the row above by different amounts; 1 row makes
# row 0 also row h - 1, 8 columns put columns 0 and w - 2 in neighbouring
# lanes.
@pytest.mark.parametrize("h,w,iters", [(9, 11, 0), (9, 11, 1), (9, 11, 2), (40, 56, 75), (3, 3, 5), (2, 2, 4),
                                       (67, 33, 150), (48, 200, 13), (540, 960, 75), (1080, 1920, 150),
                                       (17, 4, 3), (100, 64, 150), (61, 70, 19), (61, 72, 24), (1, 8, 9),
                                       (2, 4, 16), (130, 236, 40), (72, 128, 16), (120, 96, 24)])
def test_consist_out_fma(vsc, oracle, cuda, h, w, iters):
    """vsc_get_consist_out_fma equals the restatement's FMA form bit for bit,
    and the exact form (kernel_consist_out's rounding) within the stated
    tolerance: max-abs <= 2e-6 on [0, 1] images, PSNR >= 100 dB, RGBA8
    bytes differing on at most 1e-3 of the values (at least one byte: a
    value within 2e-6 of a rounding edge of the 8-bit conversion may flip)."""
    import math

    import torch

    P, A, Wt, O0 = _img(h, w), _img(h, w), _img(h, w, hi=2.0), _img(h, w)
    O = _t(O0, cuda)
    vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), iters, 0.15, 0.15, O, form="fma")
    got = O.cpu().numpy()
    ref = oracle.consist_out(P, A, Wt, iters, 0.15, 0.15, O0, form="fma")
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    exact = oracle.consist_out(P, A, Wt, iters, 0.15, 0.15, O0)
    d = np.abs(got.astype(np.float64) - exact)
    mse = float(np.mean(d * d))
    psnr = math.inf if mse == 0 else 10 * math.log10(1.0 / mse)
    flipped = oracle.float_to_rgba(got)[..., :3] != oracle.float_to_rgba(exact)[..., :3]
    flips = float(np.mean(flipped))
    print(f"fma vs exact {w}x{h} x{iters}: max-abs {d.max():.3g}, PSNR {psnr:.1f} dB, RGBA8 byte flips {flips:.2e}")
    assert d.max() <= 2e-6 and psnr >= 100.0 and int(flipped.sum()) <= max(1, int(1e-3 * flipped.size))
    # caller-provided workspace gives the same bits
    ws = torch.empty(vsc.consist_out_workspace_size(w, h, form="fma") // 4, dtype=torch.float32, device=cuda)
    O2 = _t(O0, cuda)
    vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), iters, 0.15, 0.15, O2, workspace=ws, form="fma")
    # a workspace of the exact form's size is too small for the FMA form
    if iters:
        small = torch.empty(vsc.consist_out_workspace_size(w, h) // 4, dtype=torch.float32, device=cuda)
        with pytest.raises(vsc.VscError, match="ENOMEM"):
            vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), iters, 0.15, 0.15, O2, workspace=small,
                                form="fma")
    assert np.array_equal(O2.cpu().numpy().view(np.uint32), got.view(np.uint32))


def test_consist_out_fma_single_tile_shape(vsc, cuda):
    """The FMA form has one tile shape (128 x 72 of a plane); the autotuner
    reports it without measuring."""
    assert vsc.solver_autotune(960, 544, form="fma") == 72
    assert vsc.solver_tile_rows(960, 544, form="fma") == (72, False)


def test_consist_out_zero_regions(vsc, oracle, cuda):
    """All-zero regions (black borders, zero weights) where the sign of a
    zero can differ from the oracle's: the values and the RGBA8 bytes are
    the oracle's."""
    h, w = 40, 56
    P, A, Wt, O0 = _img(h, w), _img(h, w), _img(h, w, hi=2.0), _img(h, w)
    for X in (P, A, O0):
        X[:, :9] = 0.0
        X[:12] = 0.0
    Wt[:, :20] = 0.0
    O0[:6, :6] = -0.0
    O = _t(O0, cuda)
    vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), 37, 0.15, 0.15, O)
    ref = oracle.consist_out(P, A, Wt, 37, 0.15, 0.15, O0)
    got = O.cpu().numpy()
    assert _equal_up_to_zero_sign(got, ref)
    assert np.array_equal(oracle.float_to_rgba(got), oracle.float_to_rgba(ref))


def test_bounded_wait_timeout_is_reported(vsc, oracle, cuda):
    """Failure detection without a fault: a kernel whose bounded wait runs out
    records it; the host reads VSC_ETIMEOUT once, the context stays usable."""
    import torch

    vsc.check_device()  # clear anything earlier
    vsc._check(vsc.load().vsc_selftest_bounded_wait(2000, None))
    torch.cuda.synchronize()
    with pytest.raises(vsc.VscError, match="ETIMEOUT"):
        vsc.check_device()
    vsc.check_device()  # cleared
    f = RNG.standard_normal((1, 3, 6, 6)).astype(np.float32)
    out = vsc.correlation(_t(f, cuda), _t(f, cuda), 4).cpu().numpy()
    assert np.array_equal(out, oracle.correlation(f, f, 4))


def _frames(w, h, n, seed):
    from vsc_gb300 import synth

    s = synth.SyntheticStream(w, h, seed=seed)
    return [s.frame(i) for i in range(n)]


@pytest.mark.parametrize("w,h", [(96, 64), (70, 45)])
def test_stabilizer_computed_flow_stream(vsc, oracle, cuda, w, h):
    frames = _frames(w, h, 6, seed=11)
    ref = run_oracle_stream(oracle, frames)
    st = vsc.Stabilizer(w, h)
    for i in range(3):
        st.load_frame(*frames[i])
    for k, t in enumerate(range(1, len(frames) - 1)):
        out = st.step()
        r_out, r_rgba, r_ff, r_fb = ref[k]
        assert np.array_equal(st.buffer(1).cpu().numpy(), r_ff), f"fwd flow, step {k}"
        assert np.array_equal(st.buffer(2).cpu().numpy(), r_fb), f"bwd flow, step {k}"
        assert np.array_equal(st.buffer(0).cpu().numpy(), r_out), f"stabilized, step {k}"
        assert np.array_equal(out.cpu().numpy(), r_rgba), f"rgba, step {k}"
        if t + 2 < len(frames):
            st.load_frame(*frames[t + 2])
    st.close()


@pytest.mark.parametrize("use_graphs", [True, False])
def test_stabilizer_graph_replay_side_stream(vsc, oracle, cuda, use_graphs):
    """On a non-default stream steps after the first replay captured CUDA
    graphs (one per window rotation / feedback parity); every step must still
    equal the restatement, and hyper-parameter edits must be honoured."""
    import torch

    w, h = 96, 64
    frames = _frames(w, h, 10, seed=21)
    ref = run_oracle_stream(oracle, frames[:8])
    hp = oracle.default_hyper()
    hp.num_iter = 37
    side = torch.cuda.Stream()
    st = vsc.Stabilizer(w, h, stream=side, use_graphs=use_graphs)
    for i in range(3):
        st.load_frame(*frames[i])
    outs = []
    for t in range(1, 7):
        with torch.cuda.stream(side):
            out = st.step()
        side.synchronize()
        outs.append((out.cpu().numpy(), st.buffer(0).cpu().numpy()))
        st.load_frame(*frames[t + 2])
    for k in range(6):
        assert np.array_equal(outs[k][0], ref[k][1]), f"step {k}"
        assert np.array_equal(outs[k][1], ref[k][0]), f"step {k}"
    # a hyper-parameter change takes effect on the next (re-captured) step
    st.hyper_params.num_iter = 37
    with torch.cuda.stream(side):
        out = st.step()
    side.synchronize()
    orig = [oracle.rgba_to_float(o) for o, _ in frames[6:9]]
    proc = [oracle.rgba_to_float(p) for _, p in frames[6:9]]
    ff = oracle.flow_estimate(orig[1], orig[2])
    fb = oracle.flow_estimate(orig[2], orig[1])
    _, rgba = oracle.stab_pass(orig, proc, ff, fb, outs[-1][1], hp)
    assert np.array_equal(out.cpu().numpy(), rgba)
    st.close()


def test_stabilizer_async_host_output_and_pinned_uploads(vsc, cuda):
    """Results copied back with VSC_OUT_HOST_ASYNC into pinned memory (on the
    download stream, from alternating device buffers) while the next frames
    upload from pinned memory on the copy stream equal the synchronous host
    path's bytes, each one readable after wait_output; an unknown output mode
    is rejected."""
    import torch

    w, h = 96, 64
    fr = _frames(w, h, 9, seed=31)
    pin = [(torch.from_numpy(o).pin_memory(), torch.from_numpy(p).pin_memory()) for o, p in fr]
    ref_st, st = vsc.Stabilizer(w, h), vsc.Stabilizer(w, h)
    for i in range(3):
        ref_st.load_frame(*fr[i])
        st.load_frame(pin[i][0].numpy(), pin[i][1].numpy())
    refs = []
    for t in range(6):
        out = np.empty((h, w, 4), np.uint8)
        ref_st.step(torch.from_numpy(out))
        refs.append(out.copy())
        ref_st.load_frame(*fr[t + 3])
    outs = [torch.empty((h, w, 4), dtype=torch.uint8).pin_memory() for _ in range(6)]
    for t in range(6):
        st.step(outs[t], asynchronous=True)
        if t >= 1:  # the previous step's copy, waited for alone
            st.wait_output(1)
            assert np.array_equal(outs[t - 1].numpy(), refs[t - 1]), t - 1
        st.load_frame(pin[t + 3][0].numpy(), pin[t + 3][1].numpy())
    st.synchronize()
    for t in range(6):
        assert np.array_equal(outs[t].numpy(), refs[t]), t
    with pytest.raises(vsc.VscError, match="out_on_device"):
        vsc._check(vsc.load().vsc_stabilizer_step(st._h, outs[0].data_ptr(), 3))
    st.close()
    ref_st.close()


def test_stabilizer_external_flows_host_io(vsc, oracle, cuda):
    """File mode (-f): 2-channel flows supplied per step, host frames in/out."""
    import torch

    w, h = 80, 48
    frames = _frames(w, h, 5, seed=12)
    flows = {t: (RNG.normal(0, 3, (h, w, 2)).astype(np.float32), RNG.normal(0, 3, (h, w, 2)).astype(np.float32))
             for t in range(1, 4)}
    ref = run_oracle_stream(oracle, frames, flows=flows)
    st = vsc.Stabilizer(w, h, compute_flow=False, flow_channels=2)
    for i in range(3):
        st.load_frame(*frames[i])
    for k, t in enumerate(range(1, 4)):
        st.set_flows(torch.from_numpy(flows[t][0]), torch.from_numpy(flows[t][1]))
        out = torch.empty((h, w, 4), dtype=torch.uint8)
        st.step(out)
        assert np.array_equal(out.numpy(), ref[k][1])
        if t + 2 < len(frames):
            st.load_frame(*frames[t + 2])
    with pytest.raises(vsc.VscError, match="ESTATE"):
        st.step()
    st.close()


@pytest.mark.parametrize("fc", [2, 3])
def test_flow_consistency_mask(vsc, oracle, cuda, fc):
    """Opt-in forward-backward consistency mask: the 0/1 decisions equal the
    restatement's, including pixels carried out of the frame and NaN flows."""
    h, w = 57, 83
    # a near-constant motion and its inverse are consistent (but for noise)
    ff = (np.array([2.3, -1.1, 0.0][:fc], np.float32) + RNG.normal(0, 0.1, (h, w, fc))).astype(np.float32)
    fb = (np.array([-2.3, 1.1, 0.0][:fc], np.float32) + RNG.normal(0, 0.3, (h, w, fc))).astype(np.float32)
    fb[5:15, 10:30] = RNG.normal(0, 6, (10, 20, fc))              # an inconsistent patch
    ff[0, :5, 0] = -10.0                                           # carried out of the frame
    ff[3, 3, 1] = np.nan
    ref = oracle.flow_consistency_mask(ff, fb)
    got = vsc.get_flow_consistency_mask(_t(ff, cuda), _t(fb, cuda)).cpu().numpy()
    assert np.array_equal(got, ref)
    assert 0.2 < ref.mean() < 0.98  # both outcomes occur
    assert ref[0, :5, 1].max() == 0.0 and ref[3, 3, 1] == 0.0


def test_adap_comb_masked(vsc, oracle, cuda):
    h, w = 40, 64
    base = _img(h, w)
    ims = [np.clip(base + RNG.normal(0, s, base.shape), 0, 1).astype(np.float32)
           for s in (0.0, 0.05, 0.02, 0.03, 0.02, 0.04, 0.01)]
    mask = (RNG.random((h, w, 2)) < 0.6).astype(np.float32)
    mask[:4] = RNG.random((4, w, 2)).astype(np.float32)  # soft factors multiply too
    dev = [_t(a, cuda) for a in ims]
    ain, apr = vsc.get_adap_comb_masked(*dev[:6], dev[6], _t(mask, cuda), 20.0)
    oin, opr = oracle.adap_comb_masked(*ims[:6], ims[6], mask, 20.0)
    assert np.array_equal(ain.cpu().numpy(), oin) and np.array_equal(apr.cpu().numpy(), opr)
    ones = np.ones((h, w, 2), np.float32)
    ain1, apr1 = vsc.get_adap_comb_masked(*dev[:6], dev[6], _t(ones, cuda), 20.0)
    bin_, bpr = vsc.get_adap_comb(*dev[:6], dev[6], 20.0)
    assert np.array_equal(ain1.cpu().numpy(), bin_.cpu().numpy())
    assert np.array_equal(apr1.cpu().numpy(), bpr.cpu().numpy())
    assert not np.array_equal(apr.cpu().numpy(), bpr.cpu().numpy())


@pytest.mark.parametrize("use_graphs", [False, True])
def test_stabilizer_occlusion_mask(vsc, oracle, cuda, use_graphs):
    """The opt-in mask inside the fused front end equals the restatement's
    pass with the mask; switching it off again restores the default bits."""
    import torch

    w, h = 80, 48
    frames = _frames(w, h, 6, seed=21)
    flows = {}
    for t in range(1, 5):
        ff = RNG.normal(0, 2, (h, w, 2)).astype(np.float32)
        fb = (-ff + RNG.normal(0, 0.5, ff.shape)).astype(np.float32)
        flows[t] = (ff, fb)
    ref_on = run_oracle_stream(oracle, frames, flows=flows, occlusion=True)
    ref_off = run_oracle_stream(oracle, frames, flows=flows)
    assert not np.array_equal(ref_on[0][0], ref_off[0][0])
    stream = torch.cuda.Stream()
    st = vsc.Stabilizer(w, h, compute_flow=False, flow_channels=2, stream=stream, use_graphs=use_graphs)
    st.set_occlusion_mask(True)
    for i in range(3):
        st.load_frame(*frames[i])
    for k, t in enumerate(range(1, 5)):
        st.set_flows(torch.from_numpy(flows[t][0]), torch.from_numpy(flows[t][1]))
        with torch.cuda.stream(stream):
            out = st.step()
        stream.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref_on[k][1]), k
        if t + 2 < len(frames):
            st.load_frame(*frames[t + 2])
    st.close()


def test_stabilizer_hyper_params_and_downscale(vsc, oracle, cuda):
    w, h = 128, 72
    frames = _frames(w, h, 4, seed=13)
    hp = oracle.default_hyper()
    hp.pyramid_levels, hp.num_iter, hp.gamma = 3, 40, 1.0
    ref = run_oracle_stream(oracle, frames, hp=hp, downscale=2)
    st = vsc.Stabilizer(w, h, flow_downscale=2)
    p = st.hyper_params
    p.pyramid_levels, p.num_iter, p.gamma = 3, 40, 1.0
    for i in range(3):
        st.load_frame(*frames[i])
    out = st.step().cpu().numpy()
    assert np.array_equal(st.buffer(1).cpu().numpy(), ref[0][2])
    assert np.array_equal(out, ref[0][1])
    st.close()


@pytest.mark.parametrize("w,h", [(128, 72), (134, 77)])
def test_stabilizer_fma_downscale_fused_paths(vsc, oracle, cuda, w, h):
    """FMA solver form with FLOWDOWNSCALE=2 and three pyramid levels: the
    front pass samples the coarse flows itself and each finer level's setup
    upsamples the coarser solution (no separate upsampling launches); two
    steps equal the restatement's driver loop bit for bit, and the flows
    read back on request are the upsampled ones the oracle uses."""
    frames = _frames(w, h, 5, seed=17)
    hp = oracle.default_hyper()
    hp.pyramid_levels, hp.num_iter, hp.gamma = 3, 24, 1.0
    ref = run_oracle_stream(oracle, frames, hp=hp, downscale=2, solver_form="fma")
    st = vsc.Stabilizer(w, h, flow_downscale=2, solver_form="fma")
    p = st.hyper_params
    p.pyramid_levels, p.num_iter, p.gamma = 3, 24, 1.0
    for i in range(3):
        st.load_frame(*frames[i])
    for k in range(2):
        out = st.step().cpu().numpy()
        assert np.array_equal(out, ref[k][1]), f"output, step {k}"
        assert np.array_equal(st.buffer(0).cpu().numpy(), ref[k][0]), f"stabilized, step {k}"
        assert np.array_equal(st.buffer(1).cpu().numpy(), ref[k][2]), f"fwd flow, step {k}"
        assert np.array_equal(st.buffer(2).cpu().numpy(), ref[k][3]), f"bwd flow, step {k}"
        if k + 3 < len(frames):
            st.load_frame(*frames[k + 3])
    st.close()


def test_stabilizer_state_errors(vsc, cuda):
    st = vsc.Stabilizer(32, 32)
    f = np.zeros((32, 32, 4), np.uint8)
    st.load_frame(f, f)
    with pytest.raises(vsc.VscError, match="ESTATE"):
        st.step()
    st.load_frame(f, f)
    st.load_frame(f, f)
    with pytest.raises(vsc.VscError, match="ESTATE"):
        st.load_frame(f, f)
    st.hyper_params.pyramid_levels = 9
    with pytest.raises(vsc.VscError, match="EINVAL"):
        st.step()
    st.hyper_params.pyramid_levels = 2
    st.step()
    st.close()


def test_full_hd_step_deterministic(vsc, cuda):
    """1920x1080 (the benchmark size): two stabilizers fed the same frames
    give identical outputs and internal state."""
    frames = _frames(1920, 1080, 4, seed=14)
    outs = []
    for _ in range(2):
        st = vsc.Stabilizer(1920, 1080)
        for i in range(3):
            st.load_frame(*frames[i])
        o1 = st.step()
        st.load_frame(*frames[3])
        o2 = st.step()
        outs.append((o1.cpu().numpy(), o2.cpu().numpy(), st.buffer(0).cpu().numpy()))
        st.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    assert outs[0][1][..., 3].max() == 1


@pytest.mark.parametrize("w,h,nframes", [(640, 360, 3), (1920, 1080, 4)])
def test_whole_step_equals_restatement(vsc, oracle, cuda, w, h, nframes):
    """doOneStep end to end at 640x360 (the small configuration, one step)
    and 1920x1080 (the benchmark size, two steps, so the second starts from
    the first's FP32 feedback): default hyper-parameters (2-level pyramid,
    75 iterations at half size, 150 at full size: every solve ends in a
    short launch after the unrolled 8-step ones), flows computed by the
    estimator at full size.  Forward and backward flow, FP32 state and RGBA8
    output equal the restatement's driver loop (videostabilizer.cpp:136-265
    with :118-128, :226) bit for bit (values; a zero's sign may differ)."""
    frames = _frames(w, h, nframes, seed=17)
    ref = run_oracle_stream(oracle, frames)
    st = vsc.Stabilizer(w, h)
    for i in range(3):
        st.load_frame(*frames[i])
    for k, t in enumerate(range(1, nframes - 1)):
        out = st.step().cpu().numpy()
        r_out, r_rgba, r_ff, r_fb = ref[k]
        assert np.array_equal(st.buffer(1).cpu().numpy(), r_ff), f"fwd flow, step {k}"
        assert np.array_equal(st.buffer(2).cpu().numpy(), r_fb), f"bwd flow, step {k}"
        assert _equal_up_to_zero_sign(st.buffer(0).cpu().numpy(), r_out), f"stabilized, step {k}"
        assert np.array_equal(out, r_rgba), f"rgba, step {k}"
        if t + 2 < nframes:
            st.load_frame(*frames[t + 2])
    st.close()


@pytest.mark.parametrize("w,h,nframes", [(640, 360, 3), (1920, 1080, 4), (70, 45, 4)])
def test_whole_step_fma_form_equals_restatement(vsc, oracle, cuda, w, h, nframes):
    """doOneStep with the FMA solver form equals the restatement's pass with
    that form bit for bit (the warps, mask and combination are unchanged;
    70x45 takes the plain-load kernel at both levels)."""
    frames = _frames(w, h, nframes, seed=23)
    ref = run_oracle_stream(oracle, frames, solver_form="fma")
    st = vsc.Stabilizer(w, h, solver_form="fma")
    for i in range(3):
        st.load_frame(*frames[i])
    for k, t in enumerate(range(1, nframes - 1)):
        out = st.step().cpu().numpy()
        r_out, r_rgba, _, _ = ref[k]
        assert np.array_equal(st.buffer(0).cpu().numpy().view(np.uint32), r_out.view(np.uint32)), f"step {k}"
        assert np.array_equal(out, r_rgba), f"rgba, step {k}"
        if t + 2 < nframes:
            st.load_frame(*frames[t + 2])
    st.close()


def _psnr_rgb(a, b):
    import math

    d = a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64)
    mse = float(np.mean(d * d)) / 255.0 ** 2
    return math.inf if mse == 0 else 10 * math.log10(1.0 / mse)


@pytest.mark.parametrize("solver_form", ["exact", "fma"])
def test_fast_form_quality_at_1080p(vsc, cuda, solver_form):
    """The benchmark's fast form (flow at 960x540 with bilinear upsampling,
    BF16 tensor-core correlations, the solver in either form) against the
    plain FP32 path on the same 1920x1080 stream: stabilized RGB at >= 40 dB
    PSNR in every one of six consecutive frames (the feedback carries each
    frame's difference into the next)."""
    frames = _frames(1920, 1080, 8, seed=19)
    sts = [vsc.Stabilizer(1920, 1080),
           vsc.Stabilizer(1920, 1080, flow_downscale=2, corr_dtype="bf16", solver_form=solver_form)]
    for st in sts:
        for i in range(3):
            st.load_frame(*frames[i])
    vals = []
    for t in range(1, 7):
        a, b = (st.step().cpu().numpy() for st in sts)
        vals.append(_psnr_rgb(a, b))
        if t + 2 < len(frames):
            for st in sts:
                st.load_frame(*frames[t + 2])
    for st in sts:
        st.close()
    print(f"fast form ({solver_form} solver) vs plain, PSNR per frame (dB):", [round(v, 2) for v in vals])
    assert min(vals) >= 40.0, vals


def _multistream_vs_singles(vsc, sizes, forms, fused, num_iter, upsampler=None, steps=5, levels=2,
                            solver_form="exact"):
    """Runs a MultiStream and one Stabilizer per stream (each with the
    stream's (flow_downscale, corr_dtype) form) on the same frames and
    asserts equal outputs, bit for bit, on the direct first step and on the
    graph replays that follow.  Returns the multistream's launch count."""
    import torch

    streams = [_frames(w, h, steps + 2, seed=50 + i) for i, (w, h) in enumerate(sizes)]
    side = torch.cuda.Stream()
    ms = vsc.MultiStream(sizes, flow_downscale=[f[0] for f in forms], corr_dtype=[f[1] for f in forms], stream=side)
    ms.set_fused(fused)
    if solver_form != "exact":
        ms.set_solver_form(solver_form)
    ms.hyper_params.num_iter = num_iter
    ms.hyper_params.pyramid_levels = levels
    singles = []
    for (w, h), (ds, dt) in zip(sizes, forms):
        st = vsc.Stabilizer(w, h, flow_downscale=ds, corr_dtype=dt, solver_form=solver_form)
        st.hyper_params.num_iter = num_iter
        st.hyper_params.pyramid_levels = levels
        if upsampler is not None and ds > 1:
            st.set_upsampler(upsampler)
        singles.append(st)
    if upsampler is not None:
        ms.set_upsampler(upsampler)
    for i in range(3):  # host frames: each stream uploads on its own CUDA stream
        ms.load_frames([fr[i][0] for fr in streams], [fr[i][1] for fr in streams])
        for st, fr in zip(singles, streams):
            st.load_frame(*fr[i])
    side.synchronize()
    for t in range(1, steps + 1):
        with torch.cuda.stream(side):
            outs = ms.step()
        side.synchronize()
        for k, (st, out) in enumerate(zip(singles, outs)):
            ref = st.step().cpu().numpy()
            assert np.array_equal(out.cpu().numpy(), ref), (t, k)
        if t + 2 < steps + 2:
            if t % 2:  # device frames, made ready before the call
                o = [torch.from_numpy(fr[t + 2][0]).cuda() for fr in streams]
                p = [torch.from_numpy(fr[t + 2][1]).cuda() for fr in streams]
                torch.cuda.synchronize()
                ms.load_frames(o, p)
            else:
                ms.load_frames([fr[t + 2][0] for fr in streams], [fr[t + 2][1] for fr in streams])
            for st, fr in zip(singles, streams):
                st.load_frame(*fr[t + 2])
    n = ms.last_launches
    grouped = ms.fused
    ms.close()
    for st in singles:
        st.close()
    return n, grouped


@pytest.mark.parametrize("fused,levels", [(True, 2), (False, 2), (True, 1)])
def test_multistream_equals_independent_stabilizers(vsc, cuda, fused, levels):
    """Three videos of different sizes in one multistream object, solves
    grouped into shared persistent-kernel launches or each on its own CUDA
    stream: every stream's output equals its own stabilizer's, bit for bit."""
    sizes = [(96, 64), (128, 72), (80, 48)]
    n, grouped = _multistream_vs_singles(vsc, sizes, [(1, "f32")] * 3, fused, 60, levels=levels)
    assert grouped == fused
    assert n > (3 * 20 if not fused else 8)


@pytest.mark.parametrize("fused", [True, False])
def test_multistream_fma_solver_equals_independent_stabilizers(vsc, cuda, fused):
    """The FMA solver form in a multistream step, grouped or not: every
    stream's output equals its own stabilizer's with that form."""
    sizes = [(96, 64), (128, 72), (80, 48)]
    _, grouped = _multistream_vs_singles(vsc, sizes, [(1, "f32")] * 3, fused, 45, solver_form="fma")
    assert grouped == fused


def test_multistream_mixed_forms_with_upsampler(vsc, cuda):
    """Per-stream forms in one grouped step: full-size FP32 and BF16 flows,
    and half-size flows upsampled by the learned network (odd iteration
    count, so each level's solve starts in the second buffer; three
    pyramid levels)."""
    up = vsc.Upsampler("default")
    sizes = [(96, 64), (128, 80), (160, 96), (112, 64)]
    forms = [(1, "f32"), (2, "bf16"), (2, "f32"), (1, "bf16")]
    _, grouped = _multistream_vs_singles(vsc, sizes, forms, True, 45, upsampler=up, steps=4, levels=3)
    assert grouped
    up.close()


def test_multistream_more_than_one_group(vsc, cuda):
    """18 streams: each solver launch of the grouped form covers at most 16
    images, so every level takes two launches per 8 steps; results equal the
    independent stabilizers'."""
    sizes = [(64 + 8 * (i % 5), 40 + 4 * (i % 3)) for i in range(18)]
    n, grouped = _multistream_vs_singles(vsc, sizes, [(1, "f32")] * 18, True, 40, steps=3)
    assert grouped


@pytest.mark.parametrize("num_iter", [0, 1, 9])
def test_multistream_grouped_few_iterations(vsc, cuda, num_iter):
    """Grouped solves with no iteration (the step writes the unsolved
    pyramid result), one, and nine (a level with one launch of one step)."""
    sizes = [(96, 64), (128, 72)]
    _, grouped = _multistream_vs_singles(vsc, sizes, [(1, "f32")] * 2, True, num_iter, steps=3)
    assert grouped


def test_multistream_ungroupable_size_runs_ungrouped(vsc, cuda):
    """A level width that is not a multiple of 4 (70 -> 35) keeps the step
    ungrouped, with the same results."""
    sizes = [(96, 64), (70, 45)]
    _, grouped = _multistream_vs_singles(vsc, sizes, [(1, "f32")] * 2, True, 24, steps=3)
    assert not grouped


# (alpha, beta, gamma): the kernel's fast form (32-bit taps, the exponential
# for non-positive arguments) needs alpha, beta >= 0 and |gamma| <= 1e30;
# 1e6 drives most exponents below -87.3 (the fast form's floor), gamma 2e30
# and a negative alpha take the general form
@pytest.mark.parametrize("hp", [(20.0, 30.0, 2.0), (1e6, 1e6, 2.0), (1e6, 1e6, -1e30), (20.0, 30.0, 2e30),
                                (-5.0, 30.0, 2.0)])
@pytest.mark.parametrize("fc,occ", [(3, False), (2, False), (2, True)])
def test_stab_front_equals_separate_calls(vsc, oracle, cuda, fc, occ, hp):
    """vsc_stab_front (five warps + combination + weights in one pass) equals
    the separate entry points bit for bit; with the occlusion mask, the
    restatement's masked combination."""
    h, w = 53, 77
    base = _img(h, w)
    ims = [np.clip(base + RNG.normal(0, s_, base.shape), 0, 1).astype(np.float32)
           for s_ in (0.03, 0.0, 0.02, 0.02, 0.01, 0.03, 0.01)]
    o3, p3, ls = ims[0:3], ims[3:6], ims[6]
    ff = (RNG.normal(0, 2, (h, w, fc))).astype(np.float32)
    fb = (-ff + RNG.normal(0, 0.4, ff.shape)).astype(np.float32)
    d = lambda a: _t(a, cuda)  # noqa: E731
    alpha, beta, gamma = hp
    apr, wt = vsc.stab_front([d(a) for a in o3], [d(a) for a in p3], d(ls), d(ff), d(fb), alpha, beta, gamma,
                             occlusion_mask=occ)
    warps = [oracle.stab_warp(src, fl) for src, fl in ((o3[0], fb), (p3[0], fb), (o3[2], ff), (p3[2], ff),
                                                       (ls, fb))]
    if occ:
        m = oracle.flow_consistency_mask(ff, fb)
        ain, rpr = oracle.adap_comb_masked(o3[1], p3[1], warps[0], warps[1], warps[2], warps[3], warps[4], m, alpha)
    else:
        ain, rpr = oracle.adap_comb(o3[1], p3[1], warps[0], warps[1], warps[2], warps[3], warps[4], alpha)
    rwt = oracle.consist_wt(o3[1], ain, beta, gamma)
    assert np.array_equal(apr.cpu().numpy(), rpr)
    assert np.array_equal(wt.cpu().numpy(), rwt)


@pytest.mark.parametrize("kind", ["smooth", "mixed", "shift"])
@pytest.mark.parametrize("hp", [(20.0, 30.0, 2.0), (20.0, 30.0, 2e30)])
def test_stab_front_flow_kinds(vsc, oracle, cuda, kind, hp):
    """The front pass on the flows a stream produces: smooth flows, smooth
    flows with a noisy patch, and a large uniform shift that pins taps to
    the clamped frame border.  Equal to the restatement bit for bit."""
    h, w = 75, 141
    base = _img(h, w)
    ims = [np.clip(base + RNG.normal(0, s_, base.shape), 0, 1).astype(np.float32)
           for s_ in (0.03, 0.0, 0.02, 0.02, 0.01, 0.03, 0.01)]
    o3, p3, ls = ims[0:3], ims[3:6], ims[6]
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    ff = np.zeros((h, w, 3), np.float32)
    ff[..., 0] = 3.0 * np.sin(xx / 17.0) + 0.37
    ff[..., 1] = 2.0 * np.cos(yy / 13.0) - 0.21
    if kind == "mixed":
        ff[20:45, 40:90, :2] += RNG.normal(0, 8, (25, 50, 2)).astype(np.float32)
    elif kind == "shift":
        ff[..., 0] += 60.0
        ff[..., 1] -= 40.0
    fb = (-ff + 0.3 * np.sin(xx / 11.0)[..., None]).astype(np.float32)
    d = lambda a: _t(a, cuda)  # noqa: E731
    alpha, beta, gamma = hp
    apr, wt = vsc.stab_front([d(a) for a in o3], [d(a) for a in p3], d(ls), d(ff), d(fb), alpha, beta, gamma)
    warps = [oracle.stab_warp(src, fl) for src, fl in ((o3[0], fb), (p3[0], fb), (o3[2], ff), (p3[2], ff),
                                                       (ls, fb))]
    ain, rpr = oracle.adap_comb(o3[1], p3[1], warps[0], warps[1], warps[2], warps[3], warps[4], alpha)
    assert np.array_equal(apr.cpu().numpy(), rpr)
    assert np.array_equal(wt.cpu().numpy(), oracle.consist_wt(o3[1], ain, beta, gamma))


@pytest.mark.parametrize("fc,occ", [(3, False), (2, True), (3, True)])
def test_stab_front_rgba_equals_restatement(vsc, oracle, cuda, fc, occ):
    """vsc_stab_front_rgba (taps gathered as RGBA8 words) equals the
    restatement on the converted frames bit for bit, and vsc_stab_front on
    the same converted frames; flows large enough to reach the clamped
    border taps."""
    import torch

    h, w = 61, 83
    fr = _frames(w, h, 3, seed=71)
    rgba = [o for o, _ in fr] + [p for _, p in fr]
    f = [oracle.rgba_to_float(a) for a in rgba]
    ls = np.clip(f[4] + RNG.normal(0, 0.02, f[4].shape), 0, 1).astype(np.float32)
    ff = RNG.normal(0, 6, (h, w, fc)).astype(np.float32)
    fb = (-ff + RNG.normal(0, 0.5, ff.shape)).astype(np.float32)
    d = lambda a: _t(a, cuda)  # noqa: E731
    r8 = [torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in rgba]
    apr, wt = vsc.stab_front_rgba(r8[0:3], r8[3:6], d(ls), d(ff), d(fb), 20.0, 30.0, 2.0, occlusion_mask=occ)
    fapr, fwt = vsc.stab_front([d(a) for a in f[0:3]], [d(a) for a in f[3:6]], d(ls), d(ff), d(fb), 20.0, 30.0,
                               2.0, occlusion_mask=occ)
    assert np.array_equal(apr.cpu().numpy(), fapr.cpu().numpy())
    assert np.array_equal(wt.cpu().numpy(), fwt.cpu().numpy())
    warps = [oracle.stab_warp(src, fl) for src, fl in ((f[0], fb), (f[3], fb), (f[2], ff), (f[5], ff), (ls, fb))]
    if occ:
        m = oracle.flow_consistency_mask(ff, fb)
        ain, rpr = oracle.adap_comb_masked(f[1], f[4], warps[0], warps[1], warps[2], warps[3], warps[4], m, 20.0)
    else:
        ain, rpr = oracle.adap_comb(f[1], f[4], warps[0], warps[1], warps[2], warps[3], warps[4], 20.0)
    assert np.array_equal(apr.cpu().numpy(), rpr)
    assert np.array_equal(wt.cpu().numpy(), oracle.consist_wt(f[1], ain, 30.0, 2.0))
    # misaligned frame pointer: an error, nothing launched
    bad = torch.empty(w * h * 4 + 1, dtype=torch.uint8, device=cuda)[1:].view(h, w, 4)
    with pytest.raises(vsc.VscError, match="aligned"):
        vsc.stab_front_rgba([bad, r8[1], r8[2]], r8[3:6], d(ls), d(ff), d(fb), 20.0, 30.0, 2.0)


def test_solver_autotune(vsc, oracle, cuda):
    """The tile-shape autotuner measures both persistent kernels at a size and
    keeps one; the solve at that size still equals the restatement bit for
    bit; switched off, sizes fall back to the wave model."""
    rows = vsc.solver_autotune(960, 544)
    assert rows in (32, 48)
    assert vsc.solver_tile_rows(960, 544) == (rows, True)
    assert vsc.solver_autotune(960, 544) == rows  # cached
    h, w = 544, 960
    P, A, Wt, O0 = _img(h, w), _img(h, w), _img(h, w, hi=2.0), _img(h, w)
    O = _t(O0, cuda)
    vsc.get_consist_out(_t(P, cuda), _t(A, cuda), _t(Wt, cuda), 17, 0.15, 0.15, O)
    assert np.array_equal(O.cpu().numpy(), oracle.consist_out(P, A, Wt, 17, 0.15, 0.15, O0))
    vsc.solver_set_autotune(False)
    try:
        r, tuned = vsc.solver_tile_rows(960, 544)
        assert r in (32, 48) and not tuned
        assert vsc.solver_autotune(960, 544) == r  # refused quietly: the model's choice
        assert vsc.solver_tile_rows(960, 544) == (r, False)
    finally:
        vsc.solver_set_autotune(True)
    # the stabilizer tunes its pyramid's sizes when it is created
    st = vsc.Stabilizer(200, 120)
    assert vsc.solver_tile_rows(200, 120)[1] and vsc.solver_tile_rows(100, 60)[1]
    st.close()


def test_flow_estimate_equals_restatement(vsc, oracle, cuda):
    w, h = 112, 80
    fr = _frames(w, h, 2, seed=61)
    a, b = [oracle.rgba_to_float(o) for o, _ in fr]
    ab, ba = vsc.flow_estimate(_t(a, cuda), _t(b, cuda))
    assert np.array_equal(ab.cpu().numpy(), oracle.flow_estimate(a, b))
    assert np.array_equal(ba.cpu().numpy(), oracle.flow_estimate(b, a))
