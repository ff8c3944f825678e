"""The checker itself: the C restatement (oracle/vsc_oracle.c) pinned against
the reference's own CPU custom ops compiled in place (where the reference
tree is present) and against the committed golden fixtures (everywhere)."""
from __future__ import annotations

import math

import numpy as np
import pytest

RNG = np.random.Generator(np.random.PCG64(99))


# ---- pinned to the golden fixtures made by the reference's CPU ops ----------

@pytest.mark.parametrize("i", range(5))
def test_correlation_matches_reference_fixture(oracle, golden, i):
    g = golden["ref_ops"]
    f1, f2, md = g[f"corr{i}_f1"], g[f"corr{i}_f2"], int(g[f"corr{i}_md"])
    assert np.array_equal(oracle.correlation(f1, f2, md), g[f"corr{i}_out"])
    out64 = oracle.correlation(f1.astype(np.float64), f2.astype(np.float64), md)
    assert np.array_equal(out64, g[f"corr{i}_out64"])


@pytest.mark.parametrize("i", range(3))
def test_warp_matches_reference_fixture(oracle, golden, i):
    g = golden["ref_ops"]
    x, flow = g[f"warp{i}_x"], g[f"warp{i}_flow"]
    ref = g[f"warp{i}_out"]
    # the restatement of the reference's mixed-precision arithmetic: bit-exact
    assert np.array_equal(oracle.warp_op(x, flow, "refsem"), ref)
    assert np.array_equal(oracle.warp_op(x.astype(np.float64), flow.astype(np.float64), "f64"), g[f"warp{i}_out64"])
    # the single-precision form the GPU computes: within 2^-21 of max|input|
    f32 = oracle.warp_op(x, flow, "f32")
    assert np.max(np.abs(f32 - ref)) <= 2.0 ** -21 * np.max(np.abs(x))


def test_stab_fixture_reproduced(oracle, golden):
    """The restatement gives the same bits on this machine as where the
    fixture was made (x86-64 vs aarch64, any compiler)."""
    g = golden["stab"]
    of = [oracle.rgba_to_float(a) for a in g["orig_rgba"]]
    pf = [oracle.rgba_to_float(a) for a in g["proc_rgba"]]
    ffwd = oracle.flow_estimate(of[1], of[2])
    fbwd = oracle.flow_estimate(of[2], of[1])
    assert np.array_equal(ffwd, g["flow_fwd"])
    assert np.array_equal(fbwd, g["flow_bwd"])
    out, rgba = oracle.stab_pass(of, pf, ffwd, fbwd, pf[2])
    assert np.array_equal(out, g["stab_out"])
    assert np.array_equal(rgba, g["stab_rgba"])


# ---- pinned live against the compiled reference (reference tree present) ----

def _need_ref(oracle):
    if not oracle.ref_available():
        pytest.skip("reference CPU ops not built here")


@pytest.mark.parametrize("shape,md", [((2, 7, 13, 17), 4), ((1, 32, 24, 40), 4), ((3, 2, 1, 1), 4),
                                      ((1, 5, 3, 30), 2), ((1, 1, 9, 9), 0), ((1, 6, 20, 8), 6)])
def test_correlation_live_reference(oracle, shape, md):
    _need_ref(oracle)
    f1 = RNG.standard_normal(shape).astype(np.float32)
    f2 = RNG.standard_normal(shape).astype(np.float32)
    assert np.array_equal(oracle.correlation(f1, f2, md), oracle.ref_correlation(f1, f2, md))


def test_correlation_legacy_cpu_rejected_by_reference(oracle):
    _need_ref(oracle)
    f = np.ones((1, 2, 3, 3), np.float32)
    with pytest.raises(RuntimeError, match="Legacy correlation not supported"):
        oracle.ref_correlation(f, f, 4, legacy=1)


@pytest.mark.parametrize("shape,scale,offset", [((2, 64, 64, 32), 1.0, 0.0), ((1, 5, 17, 23), 6.0, 3.0),
                                                ((1, 3, 4, 4), 10.0, 5.0), ((1, 2, 1, 7), 2.0, 1.0)])
def test_warp_live_reference(oracle, shape, scale, offset):
    _need_ref(oracle)
    x = (RNG.random(shape) * 10).astype(np.float32)
    flow = (RNG.random((shape[0], 2) + shape[2:]) * scale - offset).astype(np.float32)
    ref = oracle.ref_warp(x, flow)
    assert np.array_equal(oracle.warp_op(x, flow, "refsem"), ref)
    assert np.max(np.abs(oracle.warp_op(x, flow, "f32") - ref)) <= 2.0 ** -21 * 10


# ---- independent semantics checks ---------------------------------------------

def test_warp_matches_grid_sample_form(oracle):
    """The reference's own op test compares the Warp op with
    grid_sample(align_corners=True) * (mask >= 0.999) (model-conversion/
    test.py:99-136); here in float64 against the double-precision op."""
    torch = pytest.importorskip("torch")
    x = torch.rand((2, 6, 16, 12), dtype=torch.float64) * 10
    flow = (torch.rand((2, 2, 16, 12), dtype=torch.float64) - 0.5) * 6
    B, C, H, W = x.shape
    xx = torch.arange(0, W).view(1, -1).repeat(H, 1).view(1, 1, H, W).repeat(B, 1, 1, 1)
    yy = torch.arange(0, H).view(-1, 1).repeat(1, W).view(1, 1, H, W).repeat(B, 1, 1, 1)
    vgrid = torch.cat((xx, yy), 1).to(torch.float64) + flow
    vgrid[:, 0] = 2.0 * vgrid[:, 0] / max(W - 1, 1) - 1.0
    vgrid[:, 1] = 2.0 * vgrid[:, 1] / max(H - 1, 1) - 1.0
    vgrid = vgrid.permute(0, 2, 3, 1)
    out = torch.nn.functional.grid_sample(x, vgrid, align_corners=True)
    mask = torch.nn.functional.grid_sample(torch.ones_like(x), vgrid, align_corners=True)
    mask = (mask >= 0.999).to(torch.float64)
    alt = (out * mask).numpy()
    ours = oracle.warp_op(x.numpy(), flow.numpy(), "f64")
    # identical except where the mask sits within rounding of 0.999
    close = np.isclose(ours, alt, rtol=0, atol=1e-9)
    assert close.mean() > 0.999


def test_expf_accuracy_and_flush(oracle):
    xs = np.concatenate([np.linspace(-87.3, 88.7, 200001), RNG.uniform(-20, 5, 20000)]).astype(np.float32)
    got = np.array([oracle.lib().vo_expf(float(v)) for v in xs], np.float64)
    ref = np.exp(xs.astype(np.float64))
    ok = ref > np.finfo(np.float32).tiny
    rel = np.abs(got[ok] - ref[ok]) / ref[ok]
    assert rel.max() < 1.0 * np.finfo(np.float32).eps  # < 1 ulp
    assert oracle.lib().vo_expf(-100.0) == 0.0
    assert math.isinf(oracle.lib().vo_expf(100.0))
    assert math.isnan(oracle.lib().vo_expf(float("nan")))


def test_rgba_conversions(oracle):
    v = np.arange(256, dtype=np.uint8)
    rgba = np.stack([v, v[::-1], v, np.zeros_like(v)], -1).reshape(16, 16, 4)
    f = oracle.rgba_to_float(rgba)
    assert np.array_equal(f[..., 0].ravel(), (v.astype(np.float64) / 255.0).astype(np.float32))
    back = oracle.float_to_rgba(f)
    assert np.array_equal(back[..., :3], rgba[..., :3])
    assert np.all(back[..., 3] == 1)
    # gpuimage.cu:64 quirks: |v| taken, floor, then mod-256 wrap; NaN -> 0
    vals = np.array([[1.0, 1.01, -0.5], [2.0, np.nan, 1e30], [0.999, -1.0, 256.0 / 255.0]], np.float32).reshape(3, 1, 3)
    q = oracle.float_to_rgba(vals)[:, 0, :3]
    assert q.tolist() == [[255, 1, 127], [254, 0, 255], [254, 255, 0]]


def test_byte_to_float_single_precision_division():
    """gpuimage.cu:49 converts with a double division; for every byte value
    the single-precision quotient v / 255.0f is the same float (the kernels
    build their table that way, without FP64)."""
    v = np.arange(256)
    a = (v.astype(np.float64) / 255.0).astype(np.float32)
    b = v.astype(np.float32) / np.float32(255.0)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_bilinear_quirks(oracle):
    img = RNG.random((12, 16, 3)).astype(np.float32)
    down = oracle.bilinear(img, 8, 6)
    # source coordinate ox*Win/Wout with no half-pixel offset: even sizes decimate
    assert np.array_equal(down, img[::2, ::2])
    up = oracle.bilinear(down, 16, 12)
    assert np.array_equal(up[::2, ::2], down)
    # right tap clamped at the last column: both taps are the same pixel
    assert np.allclose(up[:, -1], up[:, -2], rtol=0, atol=1e-6)


def test_solver_semantics(oracle):
    h, w = 9, 11
    P = RNG.random((h, w, 3)).astype(np.float32)
    A = RNG.random((h, w, 3)).astype(np.float32)
    Wt = RNG.random((h, w, 3)).astype(np.float32)
    O0 = RNG.random((h, w, 3)).astype(np.float32)
    assert np.array_equal(oracle.consist_out(P, A, Wt, 0, 0.15, 0.15, O0), O0)
    # one step by hand, including the reference's neighbour rule (right
    # neighbour counted only while x+1 < w-1, bottom while y+1 < h-1)
    def lap(X):
        L = np.zeros_like(X)
        cnt = np.zeros((h, w, 1), np.float32)
        for y in range(h):
            for x in range(w):
                acc = np.zeros(3, np.float32)
                c = 0
                if x + 1 < w - 1:
                    acc = acc + X[y, x + 1]
                    c += 1
                if x - 1 >= 0:
                    acc = acc + X[y, x - 1]
                    c += 1
                if y + 1 < h - 1:
                    acc = acc + X[y + 1, x]
                    c += 1
                if y - 1 >= 0:
                    acc = acc + X[y - 1, x]
                    c += 1
                L[y, x] = acc - np.float32(c) * X[y, x]
                cnt[y, x] = c
        return L
    g = (lap(O0) - lap(P)) - Wt * (O0 - A)
    one = O0 + np.float32(0.15) * g
    assert np.array_equal(oracle.consist_out(P, A, Wt, 1, 0.15, 0.15, O0), one)
    # Jacobi: the result does not depend on traversal order -> flip symmetry
    Pf, Af, Wf, Of = (a[:, ::-1].copy() for a in (P, A, Wt, O0))
    r = oracle.consist_out(P, A, Wt, 5, 0.15, 0.15, O0)
    assert np.isfinite(r).all()


def test_flow_estimator_recovers_translation(oracle):
    from scipy.ndimage import gaussian_filter

    H, W = 128, 192
    base = np.stack([gaussian_filter(RNG.standard_normal((H + 40, W + 40)), 2.0) for _ in range(3)], -1)
    base = ((base - base.min()) / (base.max() - base.min())).astype(np.float32)
    a = base[20:20 + H, 20:20 + W].copy()
    b = base[20 - 2:20 - 2 + H, 20 - 5:20 - 5 + W].copy()  # content moved by (+5, +2)
    f = oracle.flow_estimate(a, b)
    assert abs(np.median(f[..., 0]) - 5.0) < 1.0
    assert abs(np.median(f[..., 1]) - 2.0) < 1.0
    assert np.all(f[..., 2] == 0)


def test_flow_weights_deterministic(oracle):
    w0 = oracle.flow_weights(0)
    assert w0.shape == (32, 27)
    assert np.array_equal(w0, oracle.flow_weights(0))
    assert w0.min() >= -1 and w0.max() < 1
    assert not np.array_equal(oracle.flow_weights(1)[:32], w0)
    assert [oracle.flow_level_dims(1920, 1080, l) for l in range(5)] == [
        (480, 272, 32), (240, 136, 64), (120, 68, 96), (60, 34, 128), (30, 17, 196)]


def test_stab_pass_rejects_small_pyramid(oracle):
    img = np.zeros((4, 4, 3), np.float32)
    hp = oracle.default_hyper()
    hp.pyramid_levels = 3
    with pytest.raises(ValueError):
        oracle.stab_pass([img] * 3, [img] * 3, img, img, img, hp)


def test_reference_gpu_harness_exports_its_entry_points():
    """The harness library that runs the reference's kernels exports every
    function its loader binds (checked with nm, no GPU needed)."""
    import shutil
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    lib = root / "oracle" / "_build" / "librefgpu.so"
    if not lib.exists() or shutil.which("nm") is None:
        pytest.skip("harness not built or nm missing")
    sys.path.insert(0, str(root / "oracle"))
    import ref_gpu

    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True, check=True).stdout
    names = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert set(ref_gpu.FUNCS) | {"rg_last_error"} <= names


def test_reference_gpu_harness_finds_every_kernel_in_the_cubin():
    """Each kernel the harness looks up (<length><name>, "If" for the float
    instantiation of the op templates) is a function symbol of the compiled
    reference cubin; checked on the ELF symbol table, no GPU needed."""
    import re
    import shutil
    import subprocess
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    cubin = root / "oracle" / "_ref" / "ref_kernels_exact.cubin"
    if not cubin.exists() or shutil.which("readelf") is None:
        pytest.skip("reference cubin not built or readelf missing")
    src = (root / "oracle" / "ref_gpu" / "ref_gpu_harness.cu").read_text()
    names = re.findall(r'"(\w+)"', re.search(r"kNames\[kCount\] = \{(.*?)\};", src, re.S).group(1))
    templated = re.findall(r"(true|false)", re.search(r"kTemplated\[kCount\] = \{(.*?)\};", src, re.S).group(1))
    assert len(names) == len(templated) == 11
    out = subprocess.run(["readelf", "-sW", str(cubin)], capture_output=True, text=True, check=True).stdout
    syms = [ln.split()[-1] for ln in out.splitlines() if " FUNC " in ln]
    for n, t in zip(names, templated):
        key = f"{len(n)}{n}" + ("If" if t == "true" else "")
        assert sum(key in s for s in syms) == 1, key


def test_flow_consistency_mask_semantics(oracle):
    """The opt-in forward-backward check: an exact inverse pair is consistent
    wherever the flow stays inside the frame; a flow paired with itself is
    not (unless tiny); a mask of ones leaves the combination's bits alone."""
    h, w = 30, 40
    ff = np.full((h, w, 2), [1.5, -0.5], np.float32)
    m = oracle.flow_consistency_mask(ff, -ff)
    inside = np.zeros((h, w), bool)
    inside[1:, : w - 2] = True  # x + 1.5 <= w - 1 and y - 0.5 >= 0
    assert np.array_equal(m[..., 1] == 1.0, inside)
    inside0 = np.zeros((h, w), bool)
    inside0[: h - 1, 2:] = True  # x - 1.5 >= 0 and y + 0.5 <= h - 1
    assert np.array_equal(m[..., 0] == 1.0, inside0)
    same = oracle.flow_consistency_mask(ff * 4, ff * 4)
    assert same.max() == 0.0
    rng = np.random.default_rng(3)
    ims = [rng.random((h, w, 3)).astype(np.float32) for _ in range(7)]
    a = oracle.adap_comb(*ims[:6], ims[6], 20.0)
    b = oracle.adap_comb_masked(*ims[:6], ims[6], np.ones((h, w, 2), np.float32), 20.0)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    z = oracle.adap_comb_masked(*ims[:6], ims[6], np.zeros((h, w, 2), np.float32), 20.0)
    assert np.array_equal(z[0], ims[0]) and np.array_equal(z[1], ims[1])  # no temporal weight left


def test_stab_pass_occlusion_off_is_default(oracle):
    rng = np.random.default_rng(5)
    h, w = 32, 48
    o = [rng.random((h, w, 3)).astype(np.float32) for _ in range(3)]
    p = [rng.random((h, w, 3)).astype(np.float32) for _ in range(3)]
    ff = rng.normal(0, 2, (h, w, 2)).astype(np.float32)
    fb = rng.normal(0, 2, (h, w, 2)).astype(np.float32)
    a, _ = oracle.stab_pass(o, p, ff, fb, p[2])
    b, _ = oracle.stab_pass(o, p, ff, fb, p[2], occlusion_mask=False)
    c, _ = oracle.stab_pass(o, p, ff, fb, p[2], occlusion_mask=True)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
