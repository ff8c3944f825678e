"""Frame-directory driver (the FileStabilizer equivalent) and its file
formats: PNG / PPM / JPEG images and Middlebury .flo flows.

CPU tests: the library's PNG decoder against files made here with Python's
zlib (stored, fixed and dynamic Huffman blocks; every row filter), its PNG
writer read back with Python's zlib, PPM, and .flo round trips with the
reference's error cases (flowIO.cpp:31-80, imagehelpers.cpp:42-50), and the
baseline JPEG codec: encode -> decode round trips in every mode it writes
(4:2:0 / 4:4:4 / grey, restart markers), with PSNR bars stated per mode (a
JPEG decoder's output is not fixed by the standard, so there are no exact
reference pixels), and the coding processes it refuses.
GPU tests: a whole directory stabilized through vsc_stabilize_files equals,
frame for frame and bit for bit, the reference's frame loop run over the CPU
restatement (computed flows, and flows read from a flow directory)."""
from __future__ import annotations

import struct
import zlib

import numpy as np
import pytest

RNG = np.random.Generator(np.random.PCG64(2718))


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(pix: np.ndarray, ch: int, filters) -> bytes:
    """PNG row filters (type per row) applied to h x (w*ch) uint8 rows."""
    h, stride = pix.shape
    out = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        r = pix[y].astype(np.int32)
        a = np.concatenate([np.zeros(ch, np.int32), r[:-ch]])
        c = np.concatenate([np.zeros(ch, np.int32), prev[:-ch]])
        f = filters[y % len(filters)]
        pred = [np.zeros_like(r), a, prev, (a + prev) // 2, _paeth(a, prev, c)][f]
        out.append(f)
        out += ((r - pred) & 0xFF).astype(np.uint8).tobytes()
        prev = r
    return bytes(out)


def _png_bytes(pix: np.ndarray, ctype: int, level: int, filters=(0, 1, 2, 3, 4)) -> bytes:
    h, w = pix.shape[:2]
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    raw = _filter_rows(pix.reshape(h, w * ch), ch, filters)

    def chunk(t, body):
        return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw, level)) + chunk(b"IEND", b""))


def _decode_png_py(data: bytes) -> np.ndarray:
    """Minimal reader for the RGB, filter-0 PNGs the library writes."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        t, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert zlib.crc32(t + body) & 0xFFFFFFFF == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if t == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 2
        elif t == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, w * 3 + 1)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, 3)


@pytest.mark.parametrize("ctype", [0, 2, 4, 6])
@pytest.mark.parametrize("level", [0, 1, 9])
def test_png_decoder(vsc, tmp_path, ctype, level):
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    h, w = 37, 53
    # smooth content compresses with matches (length/distance codes), noise without
    yy, xx = np.mgrid[0:h, 0:w]
    pix = ((xx * 5 + yy * 3)[..., None] + np.arange(ch) * 40) % 256
    pix[::3] = RNG.integers(0, 256, pix[::3].shape)
    pix = pix.astype(np.uint8)
    path = tmp_path / "f.png"
    path.write_bytes(_png_bytes(pix, ctype, level))
    got = vsc.read_image(path)
    want = np.empty((h, w, 4), np.uint8)
    if ch <= 2:
        want[..., :3] = pix[..., :1]
        want[..., 3] = pix[..., 1] if ch == 2 else 255
    else:
        want[..., :3] = pix[..., :3]
        want[..., 3] = pix[..., 3] if ch == 4 else 255
    assert np.array_equal(got, want)


def test_png_writer_and_large_frame(vsc, tmp_path):
    """The writer's output read by zlib; a 1920x1080 frame (several stored
    blocks) through both the library's writer and reader."""
    rgba = RNG.integers(0, 256, (1080, 1920, 4), dtype=np.uint8)
    path = tmp_path / "big.png"
    vsc.write_png(path, rgba)
    assert np.array_equal(_decode_png_py(path.read_bytes()), rgba[..., :3])
    back = vsc.read_image(path)
    assert np.array_equal(back[..., :3], rgba[..., :3]) and np.all(back[..., 3] == 255)


def test_ppm_and_unsupported_inputs(vsc, tmp_path):
    pix = RNG.integers(0, 256, (9, 14, 3), dtype=np.uint8)
    p = tmp_path / "a.ppm"
    p.write_bytes(b"P6\n# comment\n14 9\n255\n" + pix.tobytes())
    got = vsc.read_image(p)
    assert np.array_equal(got[..., :3], pix) and np.all(got[..., 3] == 255)
    j = tmp_path / "b.jpg"
    j.write_bytes(b"\xff\xd8\xff\xe0" + bytes(100))  # a JPEG start, then a zero segment length
    with pytest.raises(vsc.VscError, match="EINVAL.*corrupt JPEG"):
        vsc.read_image(j)
    bad = tmp_path / "c.png"
    data = bytearray(_png_bytes(pix, 2, 6))
    data[40] ^= 0xFF  # inside IDAT: CRC mismatch
    bad.write_bytes(bytes(data))
    with pytest.raises(vsc.VscError, match="CRC"):
        vsc.read_image(bad)


def test_flo_round_trip_and_errors(vsc, tmp_path):
    flow = RNG.normal(0, 5, (23, 31, 2)).astype(np.float32)
    p = tmp_path / "frame_000001.flo"
    vsc.write_flo(p, flow)
    raw = p.read_bytes()
    assert raw[:4] == b"PIEH" and struct.unpack("<ii", raw[4:12]) == (31, 23)
    assert np.array_equal(np.frombuffer(raw[12:], np.float32).reshape(23, 31, 2), flow)
    assert np.array_equal(vsc.read_flo(p), flow)
    import ctypes as C

    buf = np.empty((22, 31, 2), np.float32)
    assert vsc.load().vsc_read_flo(str(p).encode(), buf.ctypes.data, 31, 22) == vsc.VSC_EINVAL
    assert b"does not match" in vsc.load().vsc_last_error()
    for data, word in [(raw + b"x", "long"), (raw[:-4], "short"), (b"XXXX" + raw[4:], "tag")]:
        q = tmp_path / "bad.flo"
        q.write_bytes(data)
        with pytest.raises(vsc.VscError, match=word):
            vsc.read_flo(q)
    del C


def _smooth_rgba(h, w, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    ys, xs = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w, 3))
    for _ in range(12):
        cx, cy, sg = rng.uniform(0, w), rng.uniform(0, h), rng.uniform(3, max(4, w / 3))
        img += np.exp(-((xs - cx) ** 2 + (ys - cy) ** 2) / (2 * sg * sg))[..., None] * rng.uniform(0, 1, 3)
    out = np.full((h, w, 4), 255, np.uint8)
    out[..., :3] = np.clip(np.rint(img / img.max() * 255), 0, 255)
    return out


def _psnr8(a, b):
    import math

    m = float(np.mean((a[..., :3].astype(np.float64) - b[..., :3]) ** 2))
    return math.inf if m == 0 else 10 * math.log10(255.0 ** 2 / m)


# (quality, 4:4:4, grey, PSNR bar in dB) for smooth images
JPEG_MODES = [(95, True, False, 45.0), (75, False, False, 32.0), (90, False, True, 45.0), (40, False, False, 28.0)]


@pytest.mark.parametrize("h,w", [(48, 64), (23, 37), (1, 1), (9, 17), (130, 200)])
def test_jpeg_round_trip(vsc, tmp_path, h, w):
    img = _smooth_rgba(h, w, h * 1000 + w)
    p = tmp_path / "a.jpg"
    for q, c444, grey, bar in JPEG_MODES:
        vsc.write_jpeg(p, img, q, chroma_444=c444, grey=grey)
        assert p.read_bytes()[:4] == b"\xff\xd8\xff\xe0"
        got = vsc.read_image(p)
        assert got.shape == (h, w, 4) and (got[..., 3] == 255).all()
        ref = img
        if grey:
            y = np.clip(np.rint(0.299 * img[..., 0] + 0.587 * img[..., 1] + 0.114 * img[..., 2]), 0, 255)
            ref = np.repeat(y[..., None], 4, -1).astype(np.uint8)
            assert (got[..., 0] == got[..., 1]).all() and (got[..., 1] == got[..., 2]).all()
        assert _psnr8(got, ref) >= bar, (q, c444, grey)
        # restart markers after every MCU row change the file, not the pixels
        vsc.write_jpeg(tmp_path / "r.jpg", img, q, chroma_444=c444, grey=grey, restart_rows=True)
        if h > 16:
            assert (tmp_path / "r.jpg").read_bytes() != p.read_bytes()
        assert np.array_equal(vsc.read_image(tmp_path / "r.jpg"), got)


def test_jpeg_constant_colour(vsc, tmp_path):
    img = np.zeros((40, 56, 4), np.uint8)
    img[...] = (200, 30, 90, 255)
    vsc.write_jpeg(tmp_path / "c.jpg", img, 90)
    got = vsc.read_image(tmp_path / "c.jpg")
    assert np.abs(got[..., :3].astype(int) - img[..., :3]).max() <= 2


def test_jpeg_refused_and_corrupt(vsc, tmp_path):
    import ctypes as C

    # a progressive frame header (SOF2): refused as unsupported
    sof2 = bytes([0xFF, 0xD8, 0xFF, 0xC2, 0x00, 0x11, 0x08, 0x00, 0x10, 0x00, 0x10, 0x03,
                  0x01, 0x22, 0x00, 0x02, 0x11, 0x01, 0x03, 0x11, 0x01, 0xFF, 0xD9])
    (tmp_path / "p.jpg").write_bytes(sof2)
    with pytest.raises(vsc.VscError, match="EUNSUPPORTED.*SOF2"):
        vsc.read_image(tmp_path / "p.jpg")
    # 12-bit samples: refused
    (tmp_path / "t.jpg").write_bytes(sof2.replace(bytes([0xC2, 0x00, 0x11, 0x08]), bytes([0xC1, 0x00, 0x11, 0x0C])))
    with pytest.raises(vsc.VscError, match="EUNSUPPORTED"):
        vsc.read_image(tmp_path / "t.jpg")
    # truncated files and a corrupt segment length: errors, no crash
    good = tmp_path / "g.jpg"
    vsc.write_jpeg(good, _smooth_rgba(32, 32, 5), 80)
    data = good.read_bytes()
    for cut in (4, 30, 200, 600):
        (tmp_path / "x.jpg").write_bytes(data[:cut])
        try:
            vsc.read_image(tmp_path / "x.jpg")
        except vsc.VscError:
            pass
    bad = bytearray(data)
    bad[4:6] = b"\xff\xff"  # APP0 length past the end
    (tmp_path / "y.jpg").write_bytes(bytes(bad))
    with pytest.raises(vsc.VscError, match="EINVAL"):
        vsc.read_image(tmp_path / "y.jpg")
    # header-only size query
    w, h = C.c_int32(), C.c_int32()
    vsc._check(vsc.load().vsc_image_file_info(str(good).encode(), C.byref(w), C.byref(h)))
    assert (w.value, h.value) == (32, 32)
    with pytest.raises(vsc.VscError, match="EINVAL"):
        vsc.write_jpeg(good, _smooth_rgba(8, 8, 1), 0)


def _write_stream(vsc, tmp_path, frames):
    od, pd = tmp_path / "orig", tmp_path / "proc"
    od.mkdir()
    pd.mkdir()
    for i, (o, p) in enumerate(frames):
        vsc.write_png(od / f"{i:06d}.png", o)
        vsc.write_png(pd / f"frame{i:04d}.png", p)
    return od, pd


@pytest.mark.gpu
def test_stabilize_files_computed_flow(vsc, oracle, cuda, tmp_path):
    from oracle_driver import run_oracle_stream
    from vsc_gb300 import synth

    w, h = 96, 64
    s = synth.SyntheticStream(w, h, seed=41)
    frames = [s.frame(i) for i in range(6)]
    frames = [(o.copy(), p.copy()) for o, p in frames]
    for o, p in frames:  # PNG has no alpha channel here: the API sees alpha 255
        o[..., 3] = 255
        p[..., 3] = 255
    od, pd = _write_stream(vsc, tmp_path, frames)
    out = tmp_path / "out"
    assert vsc.stabilize_files(od, pd, out) == 6
    files = sorted(out.iterdir())
    assert [f.name for f in files] == [f"{i:06d}.png" for i in range(6)]
    ref = run_oracle_stream(oracle, frames)
    for t in range(1, 5):
        assert np.array_equal(vsc.read_image(out / f"{t:06d}.png")[..., :3], ref[t - 1][1][..., :3]), t
    # first and last frames: the processed frames through the float conversion and back
    for idx in (0, 5):
        back = oracle.float_to_rgba(oracle.rgba_to_float(frames[idx][1]))
        assert np.array_equal(vsc.read_image(out / f"{idx:06d}.png")[..., :3], back[..., :3])


@pytest.mark.gpu
def test_stabilize_files_jpeg_frames(vsc, oracle, cuda, tmp_path):
    """A frame directory of JPEG files, as the reference reads them, stabilized
    into .jpg outputs as the reference writes them: the stabilized frames
    equal the restatement's loop over the decoded input frames (bit for bit
    before the output encoding); the written .jpg files decode to within
    35 dB of those frames."""
    from oracle_driver import run_oracle_stream
    from vsc_gb300 import synth

    w, h = 96, 64
    s = synth.SyntheticStream(w, h, seed=45)
    frames = [tuple(a.copy() for a in s.frame(i)) for i in range(5)]
    od, pd = tmp_path / "orig", tmp_path / "proc"
    od.mkdir()
    pd.mkdir()
    for i, (o, p) in enumerate(frames):
        vsc.write_jpeg(od / f"{i:06d}.jpg", o, 92)
        vsc.write_jpeg(pd / f"frame{i:04d}.jpeg", p, 92)
    decoded = [(vsc.read_image(od / f"{i:06d}.jpg"), vsc.read_image(pd / f"frame{i:04d}.jpeg")) for i in range(5)]
    ref = run_oracle_stream(oracle, decoded)
    out_png, out_jpg = tmp_path / "out_png", tmp_path / "out_jpg"
    assert vsc.stabilize_files(od, pd, out_png) == 5
    assert vsc.stabilize_files(od, pd, out_jpg, jpeg_quality=90) == 5
    assert sorted(f.name for f in out_jpg.iterdir()) == [f"{i:06d}.jpg" for i in range(5)]
    for t in range(1, 4):
        assert np.array_equal(vsc.read_image(out_png / f"{t:06d}.png")[..., :3], ref[t - 1][1][..., :3]), t
        assert _psnr8(vsc.read_image(out_jpg / f"{t:06d}.jpg"), ref[t - 1][1]) >= 35.0, t


@pytest.mark.gpu
def test_stabilize_files_flow_directory(vsc, oracle, cuda, tmp_path):
    """-f mode: frame_<i+1>.flo is the forward flow of frame i,
    frame_<i>_bwd.flo its backward flow."""
    from oracle_driver import run_oracle_stream
    from vsc_gb300 import synth

    w, h = 80, 48
    s = synth.SyntheticStream(w, h, seed=43)
    frames = [tuple(a.copy() for a in s.frame(i)) for i in range(5)]
    for o, p in frames:
        o[..., 3] = 255
        p[..., 3] = 255
    od, pd = _write_stream(vsc, tmp_path, frames)
    fd = tmp_path / "flow"
    fd.mkdir()
    flows = {}
    for i in range(1, 4):
        ff = RNG.normal(0, 2, (h, w, 2)).astype(np.float32)
        fb = RNG.normal(0, 2, (h, w, 2)).astype(np.float32)
        vsc.write_flo(fd / f"frame_{i + 1:06d}.flo", ff)
        vsc.write_flo(fd / f"frame_{i:06d}_bwd.flo", fb)
        flows[i] = (ff, fb)
    out = tmp_path / "out"
    hp = vsc.default_hyper_params()
    hp.num_iter = 60
    assert vsc.stabilize_files(od, pd, out, flow_dir=fd, hyper=hp) == 5
    ohp = oracle.default_hyper()
    ohp.num_iter = 60
    ref = run_oracle_stream(oracle, frames, flows=flows, hp=ohp)
    for t in range(1, 4):
        assert np.array_equal(vsc.read_image(out / f"{t:06d}.png")[..., :3], ref[t - 1][1][..., :3]), t
    # a missing flow file is an error with its path
    (fd / "frame_000002_bwd.flo").unlink()
    with pytest.raises(vsc.VscError, match="frame_000002_bwd.flo"):
        vsc.stabilize_files(od, pd, tmp_path / "out2", flow_dir=fd)
