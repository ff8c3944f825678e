// Baseline JPEG (ITU-T T.81) for the frame-directory driver: the reference
// reads *.jpg frames and writes its stabilized frames as .jpg through Qt
// (stabilizefiles.cpp:72-106).  Written here from the standard, host code, no
// library dependency.
//   * decoder: sequential DCT with Huffman coding (SOF0 / SOF1), 8-bit
//     samples, one component (grey) or three (YCbCr, or RGB when an Adobe
//     APP14 segment says so), any sampling factors of 1..4, interleaved and
//     non-interleaved scans, restart markers.  Progressive, lossless and
//     arithmetic-coded files are reported as unsupported.  Each block goes
//     through a separable floating-point inverse DCT; subsampled chroma is
//     replicated to the full grid; YCbCr -> RGB with the JFIF equations.  A
//     decoder's output is not fixed by the standard (inverse-DCT rounding,
//     chroma upsampling), so pixels can differ by a few levels from another
//     decoder's.
//   * encoder: JFIF, 4:2:0 (2x2 luma blocks per MCU, the common default) or
//     4:4:4, the standard's example quantisation tables (Annex K.1) scaled
//     by an IJG-style quality in 1..100, the standard's example Huffman
//     tables (Annex K.3), optional restart markers after every MCU row.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "vsc.h"

namespace vsc {
vsc_status set_error(vsc_status s, const char* fmt, ...);

namespace {

// zig-zag position -> natural (row-major) index, built by walking the
// anti-diagonals in alternating directions
struct ZigZag {
    int nat[64];
    ZigZag()
    {
        int k = 0;
        for (int s = 0; s < 15; ++s) {
            if (s % 2 == 0) {  // upwards: row from high to low
                for (int r = std::min(s, 7); r >= 0 && s - r < 8; --r)
                    nat[k++] = r * 8 + (s - r);
            } else {
                for (int c = std::min(s, 7); c >= 0 && s - c < 8; --c)
                    nat[k++] = (s - c) * 8 + c;
            }
        }
    }
};
const ZigZag kZZ;

// cos((2x + 1) u pi / 16) * C(u) / 2, C(0) = 1/sqrt(2)
struct CosTable {
    float c[8][8];  // [x][u]
    CosTable()
    {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                c[x][u] = static_cast<float>((u == 0 ? std::sqrt(0.5) : 1.0) *
                                             std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0) / 2.0);
    }
};
const CosTable kCos;

// in: 64 dequantised coefficients (natural order); out: 64 samples, level-shifted, rounded, clamped
void idct8x8(const float* in, uint8_t* out, int stride)
{
    float tmp[64];
    for (int y = 0; y < 8; ++y)  // rows: along u for each v
        for (int x = 0; x < 8; ++x) {
            float s = 0.0f;
            for (int u = 0; u < 8; ++u)
                s += kCos.c[x][u] * in[y * 8 + u];
            tmp[y * 8 + x] = s;
        }
    for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
            float s = 0.0f;
            for (int v = 0; v < 8; ++v)
                s += kCos.c[y][v] * tmp[v * 8 + x];
            const float val = std::nearbyint(s + 128.0f);
            out[y * stride + x] = static_cast<uint8_t>(val < 0.0f ? 0.0f : (val > 255.0f ? 255.0f : val));
        }
}

// in: 64 samples (level-shifted floats); out: 64 coefficients (natural order)
void fdct8x8(const float* in, float* out)
{
    float tmp[64];
    for (int y = 0; y < 8; ++y)
        for (int u = 0; u < 8; ++u) {
            float s = 0.0f;
            for (int x = 0; x < 8; ++x)
                s += kCos.c[x][u] * in[y * 8 + x];
            tmp[y * 8 + u] = s;
        }
    for (int u = 0; u < 8; ++u)
        for (int v = 0; v < 8; ++v) {
            float s = 0.0f;
            for (int y = 0; y < 8; ++y)
                s += kCos.c[y][v] * tmp[y * 8 + u];
            out[v * 8 + u] = s;
        }
}

uint8_t clamp8(float v)
{
    const float r = std::nearbyint(v);
    return static_cast<uint8_t>(r < 0.0f ? 0.0f : (r > 255.0f ? 255.0f : r));
}

// ---- decoder ---------------------------------------------------------------------
struct Huff {
    bool present = false;
    // canonical code: for each length l, codes [mincode[l], maxcode[l]] map to vals[valptr[l] + code - mincode[l]]
    int mincode[17] = {}, maxcode[17] = {}, valptr[17] = {};
    uint8_t vals[256] = {};
};

bool build_huff(const uint8_t* counts, const uint8_t* vals, int nvals, Huff* h)
{
    int code = 0, k = 0;
    for (int l = 1; l <= 16; ++l) {
        h->valptr[l] = k;
        h->mincode[l] = code;
        code += counts[l - 1];
        k += counts[l - 1];
        h->maxcode[l] = counts[l - 1] ? code - 1 : -1;
        if (code > (1 << l))  // more codes than this length can hold
            return false;
        code <<= 1;
    }
    if (k != nvals || k > 256)
        return false;
    std::memcpy(h->vals, vals, static_cast<size_t>(k));
    h->present = true;
    return true;
}

struct Comp {
    int id = 0, hs = 1, vs = 1, tq = 0;
    int td = 0, ta = 0;            // Huffman tables of the current scan
    int bw = 0, bh = 0;            // blocks across / down (padded to whole MCUs)
    int pred = 0;                  // DC predictor
    std::vector<uint8_t> samples;  // bw*8 x bh*8
};

struct Reader {
    const uint8_t* d;
    size_t n, pos = 0;
    uint32_t acc = 0;
    int nbits = 0;
    bool marker_hit = false;
    Reader(const uint8_t* d_, size_t n_, size_t p) : d(d_), n(n_), pos(p) {}

    // one bit of entropy-coded data; zeros past a marker or the end (the
    // caller's block counts decide what is valid)
    int bit()
    {
        if (nbits == 0) {
            uint8_t b = 0;
            if (!marker_hit && pos < n) {
                b = d[pos];
                if (b == 0xFF) {
                    if (pos + 1 < n && d[pos + 1] == 0x00) {
                        pos += 2;
                    } else {
                        marker_hit = true;  // a marker: stop consuming
                        b = 0;
                    }
                } else {
                    ++pos;
                }
            }
            acc = b;
            nbits = 8;
        }
        --nbits;
        return (acc >> nbits) & 1;
    }
    int bits(int k)
    {
        int v = 0;
        for (int i = 0; i < k; ++i)
            v = (v << 1) | bit();
        return v;
    }
    // restart: drop the partial byte, expect RSTn
    bool restart(int expect)
    {
        nbits = 0;
        if (!marker_hit) {
            // skip to the marker (fill bits are all in the dropped byte)
            while (pos < n && d[pos] != 0xFF)
                ++pos;
        }
        if (pos + 1 >= n || d[pos] != 0xFF || d[pos + 1] != (0xD0 | (expect & 7)))
            return false;
        pos += 2;
        marker_hit = false;
        return true;
    }
};

int decode_huff(Reader& r, const Huff& h)
{
    int code = 0;
    for (int l = 1; l <= 16; ++l) {
        code = (code << 1) | r.bit();
        if (h.maxcode[l] >= 0 && code <= h.maxcode[l] && code >= h.mincode[l])
            return h.vals[h.valptr[l] + code - h.mincode[l]];
    }
    return -1;
}

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

bool decode_block(Reader& r, Comp& c, const Huff* dc, const Huff* ac, const uint16_t* q, uint8_t* out, int stride)
{
    float coef[64] = {};
    const int t = decode_huff(r, dc[c.td]);
    if (t < 0 || t > 11)
        return false;
    c.pred += extend(r.bits(t), t);
    coef[0] = static_cast<float>(c.pred * q[0]);
    for (int k = 1; k < 64;) {
        const int rs = decode_huff(r, ac[c.ta]);
        if (rs < 0)
            return false;
        const int run = rs >> 4, s = rs & 15;
        if (s == 0) {
            if (run == 15) {
                k += 16;
                continue;
            }
            break;  // end of block
        }
        k += run;
        if (k > 63)
            return false;
        coef[kZZ.nat[k]] = static_cast<float>(extend(r.bits(s), s) * q[k]);
        ++k;
    }
    idct8x8(coef, out, stride);
    return true;
}

}  // namespace

// d: the whole file.  rgba: w x h x 4 (alpha 255) unless header_only.
vsc_status jpeg_decode(const uint8_t* d, size_t n, const char* path, int* w_out, int* h_out,
    std::vector<uint8_t>* rgba, bool header_only)
{
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8)
        return set_error(VSC_EINVAL, "%s: not a JPEG file", path);
    uint16_t qt[4][64] = {};
    bool qt_ok[4] = {};
    Huff dc[4], ac[4];
    std::vector<Comp> comps;
    int W = 0, H = 0, hmax = 1, vmax = 1, restart_interval = 0, adobe_transform = -1;
    bool frame = false;
    int scans = 0;
    size_t pos = 2;
    auto seg_len = [&](size_t at) -> int {
        return at + 1 < n ? (d[at] << 8) | d[at + 1] : -1;
    };
    while (pos + 4 <= n) {
        if (d[pos] != 0xFF)
            return set_error(VSC_EINVAL, "%s: corrupt JPEG (no marker at byte %zu)", path, pos);
        const int m = d[pos + 1];
        if (m == 0xFF) {  // fill byte
            ++pos;
            continue;
        }
        pos += 2;
        if (m == 0xD9)  // EOI
            break;
        if (m >= 0xD0 && m <= 0xD7)
            continue;
        const int len = seg_len(pos);
        if (len < 2 || pos + static_cast<size_t>(len) > n)
            return set_error(VSC_EINVAL, "%s: corrupt JPEG (segment length)", path);
        const uint8_t* s = d + pos + 2;
        const int sl = len - 2;
        if (m == 0xDB) {  // DQT
            for (int i = 0; i < sl;) {
                const int pq = s[i] >> 4, tq = s[i] & 15;
                if (tq > 3 || pq > 1 || i + 1 + 64 * (pq + 1) > sl)
                    return set_error(VSC_EINVAL, "%s: corrupt JPEG (DQT)", path);
                for (int k = 0; k < 64; ++k)
                    qt[tq][k] = pq ? static_cast<uint16_t>((s[i + 1 + 2 * k] << 8) | s[i + 2 + 2 * k])
                                   : s[i + 1 + k];
                qt_ok[tq] = true;
                i += 1 + 64 * (pq + 1);
            }
        } else if (m == 0xC4) {  // DHT
            for (int i = 0; i < sl;) {
                if (i + 17 > sl)
                    return set_error(VSC_EINVAL, "%s: corrupt JPEG (DHT)", path);
                const int tc = s[i] >> 4, th = s[i] & 15;
                int nv = 0;
                for (int l = 0; l < 16; ++l)
                    nv += s[i + 1 + l];
                if (tc > 1 || th > 3 || i + 17 + nv > sl ||
                    !build_huff(s + i + 1, s + i + 17, nv, tc ? &ac[th] : &dc[th]))
                    return set_error(VSC_EINVAL, "%s: corrupt JPEG (DHT)", path);
                i += 17 + nv;
            }
        } else if (m == 0xC0 || m == 0xC1) {  // SOF0 / SOF1: sequential DCT, Huffman
            if (sl < 6 || s[0] != 8)
                return set_error(VSC_EUNSUPPORTED, "%s: JPEG with %d-bit samples (8 is supported)", path,
                    sl > 0 ? s[0] : 0);
            H = (s[1] << 8) | s[2];
            W = (s[3] << 8) | s[4];
            const int nc = s[5];
            if (W < 1 || H < 1 || (nc != 1 && nc != 3) || sl < 6 + 3 * nc)
                return set_error(VSC_EUNSUPPORTED, "%s: JPEG of %dx%d with %d components (1 or 3 are supported)",
                    path, W, H, nc);
            comps.assign(nc, Comp{});
            for (int c = 0; c < nc; ++c) {
                comps[c].id = s[6 + 3 * c];
                comps[c].hs = s[7 + 3 * c] >> 4;
                comps[c].vs = s[7 + 3 * c] & 15;
                comps[c].tq = s[8 + 3 * c];
                if (comps[c].hs < 1 || comps[c].hs > 4 || comps[c].vs < 1 || comps[c].vs > 4 || comps[c].tq > 3)
                    return set_error(VSC_EINVAL, "%s: corrupt JPEG (SOF)", path);
                hmax = std::max(hmax, comps[c].hs);
                vmax = std::max(vmax, comps[c].vs);
            }
            frame = true;
            if (header_only)
                break;
            const int mcux = (W + 8 * hmax - 1) / (8 * hmax), mcuy = (H + 8 * vmax - 1) / (8 * vmax);
            for (Comp& c : comps) {
                c.bw = mcux * c.hs;
                c.bh = mcuy * c.vs;
                c.samples.assign(static_cast<size_t>(c.bw) * 8 * c.bh * 8, 0);
            }
        } else if ((m >= 0xC2 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            return set_error(VSC_EUNSUPPORTED, "%s: JPEG coding process SOF%d (baseline / extended sequential "
                "Huffman are supported)", path, m - 0xC0);
        } else if (m == 0xDD) {  // DRI
            if (sl < 2)
                return set_error(VSC_EINVAL, "%s: corrupt JPEG (DRI)", path);
            restart_interval = (s[0] << 8) | s[1];
        } else if (m == 0xEE) {  // APP14: Adobe colour transform flag
            if (sl >= 12 && std::memcmp(s, "Adobe", 5) == 0)
                adobe_transform = s[11];
        } else if (m == 0xDA) {  // SOS
            if (!frame)
                return set_error(VSC_EINVAL, "%s: corrupt JPEG (scan before frame header)", path);
            const int ns = sl > 0 ? s[0] : 0;
            if (ns < 1 || ns > static_cast<int>(comps.size()) || sl < 1 + 2 * ns + 3)
                return set_error(VSC_EINVAL, "%s: corrupt JPEG (SOS)", path);
            std::vector<Comp*> sc;
            for (int i = 0; i < ns; ++i) {
                Comp* c = nullptr;
                for (Comp& k : comps)
                    if (k.id == s[1 + 2 * i])
                        c = &k;
                if (!c)
                    return set_error(VSC_EINVAL, "%s: corrupt JPEG (scan component)", path);
                c->td = s[2 + 2 * i] >> 4;
                c->ta = s[2 + 2 * i] & 15;
                if (c->td > 3 || c->ta > 3 || !dc[c->td].present || !ac[c->ta].present || !qt_ok[c->tq])
                    return set_error(VSC_EINVAL, "%s: JPEG scan uses a missing table", path);
                c->pred = 0;
                sc.push_back(c);
            }
            const int ss = s[1 + 2 * ns], se = s[2 + 2 * ns], ahal = s[3 + 2 * ns];
            if (ss != 0 || se != 63 || ahal != 0)
                return set_error(VSC_EUNSUPPORTED, "%s: JPEG scan with spectral selection (progressive)", path);
            Reader r(d, n, pos + len);
            // MCUs of the scan: interleaved (several components) or one block per MCU
            int mcux, mcuy;
            if (ns == 1) {
                mcux = (((W * sc[0]->hs + hmax - 1) / hmax) + 7) / 8;
                mcuy = (((H * sc[0]->vs + vmax - 1) / vmax) + 7) / 8;
            } else {
                mcux = (W + 8 * hmax - 1) / (8 * hmax);
                mcuy = (H + 8 * vmax - 1) / (8 * vmax);
            }
            int since_restart = 0, rst = 0;
            for (int my = 0; my < mcuy; ++my)
                for (int mx = 0; mx < mcux; ++mx) {
                    if (restart_interval && since_restart == restart_interval) {
                        if (!r.restart(rst++))
                            return set_error(VSC_EINVAL, "%s: corrupt JPEG (restart marker)", path);
                        for (Comp* c : sc)
                            c->pred = 0;
                        since_restart = 0;
                    }
                    for (Comp* c : sc) {
                        const int stride = c->bw * 8;
                        const int nby = ns == 1 ? 1 : c->vs, nbx = ns == 1 ? 1 : c->hs;
                        for (int by = 0; by < nby; ++by)
                            for (int bx = 0; bx < nbx; ++bx) {
                                const int X = (ns == 1 ? mx : mx * c->hs + bx), Y = (ns == 1 ? my : my * c->vs + by);
                                uint8_t* out = &c->samples[(static_cast<size_t>(Y) * 8) * stride + X * 8];
                                if (!decode_block(r, *c, dc, ac, qt[c->tq], out, stride))
                                    return set_error(VSC_EINVAL, "%s: corrupt JPEG (entropy-coded data)", path);
                            }
                    }
                    ++since_restart;
                }
            ++scans;
            // continue after the entropy-coded data: the next marker
            size_t p = r.pos;
            while (p + 1 < n && !(d[p] == 0xFF && d[p + 1] != 0x00 && !(d[p + 1] >= 0xD0 && d[p + 1] <= 0xD7)))
                ++p;
            pos = p;
            continue;
        }
        pos += static_cast<size_t>(len);
    }
    if (!frame)
        return set_error(VSC_EINVAL, "%s: JPEG without a frame header", path);
    *w_out = W;
    *h_out = H;
    if (header_only)
        return VSC_OK;
    if (!scans)
        return set_error(VSC_EINVAL, "%s: JPEG without image data", path);
    rgba->resize(static_cast<size_t>(W) * H * 4);
    const bool ycc = comps.size() == 3 && adobe_transform != 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float v[3];
            for (size_t c = 0; c < comps.size(); ++c) {
                const Comp& k = comps[c];
                const int sx = x * k.hs / hmax, sy = y * k.vs / vmax;  // replicated to the full grid
                v[c] = k.samples[static_cast<size_t>(sy) * k.bw * 8 + sx];
            }
            uint8_t* o = &(*rgba)[(static_cast<size_t>(y) * W + x) * 4];
            if (comps.size() == 1) {
                o[0] = o[1] = o[2] = static_cast<uint8_t>(v[0]);
            } else if (ycc) {  // JFIF
                const float cb = v[1] - 128.0f, cr = v[2] - 128.0f;
                o[0] = clamp8(v[0] + 1.402f * cr);
                o[1] = clamp8(v[0] - 0.344136f * cb - 0.714136f * cr);
                o[2] = clamp8(v[0] + 1.772f * cb);
            } else {
                o[0] = static_cast<uint8_t>(v[0]);
                o[1] = static_cast<uint8_t>(v[1]);
                o[2] = static_cast<uint8_t>(v[2]);
            }
            o[3] = 255;
        }
    return VSC_OK;
}

// ---- encoder ---------------------------------------------------------------------
namespace {

// Annex K.1: example luminance and chrominance quantisation tables (natural order)
const uint8_t kLumQ[64] = {16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57,
    69, 56, 14, 17, 22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64, 81, 104, 113, 92, 49,
    64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kChrQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99, 24, 26, 56, 99, 99, 99,
    99, 99, 47, 66, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
    99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

// Annex K.3: example Huffman tables (code counts per length 1..16, symbols)
const uint8_t kDcLumBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kDcChrBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kAcLumBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kAcLumVals[162] = {0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51,
    0x61, 0x07, 0x22, 0x71, 0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24,
    0x33, 0x62, 0x72, 0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35,
    0x36, 0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58,
    0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3, 0xa4,
    0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3, 0xc4, 0xc5,
    0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2, 0xe3, 0xe4, 0xe5,
    0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
const uint8_t kAcChrBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
const uint8_t kAcChrVals[162] = {0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07,
    0x61, 0x71, 0x13, 0x22, 0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15,
    0x62, 0x72, 0xd1, 0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a,
    0x35, 0x36, 0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57,
    0x58, 0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2,
    0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3,
    0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe2, 0xe3, 0xe4,
    0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

// code and length per symbol of a canonical table
struct EncHuff {
    uint16_t code[256] = {};
    uint8_t len[256] = {};
    bool has[256] = {};
};

EncHuff enc_huff(const uint8_t* bits, const uint8_t* vals)
{
    EncHuff e;
    int code = 0, k = 0;
    for (int l = 1; l <= 16; ++l) {
        for (int i = 0; i < bits[l - 1]; ++i, ++k) {
            e.code[vals[k]] = static_cast<uint16_t>(code++);
            e.len[vals[k]] = static_cast<uint8_t>(l);
            e.has[vals[k]] = true;
        }
        code <<= 1;
    }
    return e;
}

struct BitWriter {
    std::vector<uint8_t>& out;
    uint32_t acc = 0;
    int nbits = 0;
    explicit BitWriter(std::vector<uint8_t>& o) : out(o) {}
    void put(uint32_t v, int n)
    {
        for (int i = n - 1; i >= 0; --i) {
            acc = (acc << 1) | ((v >> i) & 1);
            if (++nbits == 8) {
                out.push_back(static_cast<uint8_t>(acc));
                if (acc == 0xFF)
                    out.push_back(0x00);  // byte stuffing
                acc = 0;
                nbits = 0;
            }
        }
    }
    void flush()  // pad with ones to a byte boundary
    {
        while (nbits)
            put(1, 1);
    }
};

int category(int v)
{
    int a = v < 0 ? -v : v, s = 0;
    while (a) {
        ++s;
        a >>= 1;
    }
    return s;
}

void put_value(BitWriter& bw, int v, int s)
{
    if (s)
        bw.put(static_cast<uint32_t>(v < 0 ? v + (1 << s) - 1 : v), s);
}

void encode_block(BitWriter& bw, const float* samples, const uint8_t* q, const EncHuff& dc, const EncHuff& ac,
    int* pred)
{
    float coef[64];
    fdct8x8(samples, coef);
    int z[64];
    for (int k = 0; k < 64; ++k) {  // baseline: at most 11-bit DC differences, 10-bit AC values
        const int v = static_cast<int>(std::nearbyint(coef[kZZ.nat[k]] / q[k]));
        z[k] = std::max(-1023, std::min(1023, v));
    }
    const int diff = z[0] - *pred;
    *pred = z[0];
    const int s0 = category(diff);
    bw.put(dc.code[s0], dc.len[s0]);
    put_value(bw, diff, s0);
    int run = 0;
    for (int k = 1; k < 64; ++k) {
        if (z[k] == 0) {
            ++run;
            continue;
        }
        while (run > 15) {
            bw.put(ac.code[0xF0], ac.len[0xF0]);
            run -= 16;
        }
        const int s = category(z[k]);
        const int rs = (run << 4) | s;
        bw.put(ac.code[rs], ac.len[rs]);
        put_value(bw, z[k], s);
        run = 0;
    }
    if (run)
        bw.put(ac.code[0x00], ac.len[0x00]);
}

void put16(std::vector<uint8_t>& v, int x)
{
    v.push_back(static_cast<uint8_t>(x >> 8));
    v.push_back(static_cast<uint8_t>(x));
}

}  // namespace

// flags: bit 0 = 4:4:4 (else 4:2:0), bit 1 = a restart marker after every MCU
// row, bit 2 = one grey component (the luma)
vsc_status jpeg_encode(const uint8_t* rgba, int W, int H, int quality, int flags, std::vector<uint8_t>* out)
{
    if (W < 1 || H < 1 || W > 65535 || H > 65535 || quality < 1 || quality > 100)
        return set_error(VSC_EINVAL, "jpeg: size %dx%d or quality %d out of range", W, H, quality);
    const bool grey = (flags & 4) != 0;
    const bool s444 = (flags & 1) || grey, rst = (flags & 2) != 0;
    const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
    uint8_t q[2][64];
    for (int k = 0; k < 64; ++k) {  // zig-zag order, as DQT stores them
        const int l = (kLumQ[kZZ.nat[k]] * scale + 50) / 100, c = (kChrQ[kZZ.nat[k]] * scale + 50) / 100;
        q[0][k] = static_cast<uint8_t>(std::min(255, std::max(1, l)));
        q[1][k] = static_cast<uint8_t>(std::min(255, std::max(1, c)));
    }
    const EncHuff dcl = enc_huff(kDcLumBits, kDcVals), dcc = enc_huff(kDcChrBits, kDcVals);
    const EncHuff acl = enc_huff(kAcLumBits, kAcLumVals), acc = enc_huff(kAcChrBits, kAcChrVals);
    for (int s = 0; s < 16; ++s)  // every (run, size) symbol the encoder can emit has a code
        for (int sz = 1; sz <= 10; ++sz)
            if (!acl.has[(s << 4) | sz] || !acc.has[(s << 4) | sz])
                return set_error(VSC_EINVAL, "jpeg: incomplete AC Huffman table");
    std::vector<uint8_t>& o = *out;
    o.clear();
    o.insert(o.end(), {0xFF, 0xD8, 0xFF, 0xE0, 0x00, 0x10, 'J', 'F', 'I', 'F', 0x00, 0x01, 0x01, 0x00, 0x00, 0x01,
                          0x00, 0x01, 0x00, 0x00});
    for (int t = 0; t < 2; ++t) {
        o.insert(o.end(), {0xFF, 0xDB, 0x00, 0x43, static_cast<uint8_t>(t)});
        o.insert(o.end(), q[t], q[t] + 64);
    }
    const int hs = s444 ? 1 : 2, vs = s444 ? 1 : 2;
    o.insert(o.end(), {0xFF, 0xC0, 0x00, static_cast<uint8_t>(grey ? 0x0B : 0x11), 0x08});
    put16(o, H);
    put16(o, W);
    if (grey)
        o.insert(o.end(), {0x01, 0x01, 0x11, 0x00});
    else
        o.insert(o.end(), {0x03, 0x01, static_cast<uint8_t>((hs << 4) | vs), 0x00, 0x02, 0x11, 0x01, 0x03, 0x11, 0x01});
    auto dht = [&](int tc, int th, const uint8_t* bits, const uint8_t* vals, int nv) {
        o.insert(o.end(), {0xFF, 0xC4});
        put16(o, 2 + 1 + 16 + nv);
        o.push_back(static_cast<uint8_t>((tc << 4) | th));
        o.insert(o.end(), bits, bits + 16);
        o.insert(o.end(), vals, vals + nv);
    };
    dht(0, 0, kDcLumBits, kDcVals, 12);
    dht(1, 0, kAcLumBits, kAcLumVals, 162);
    if (!grey) {
        dht(0, 1, kDcChrBits, kDcVals, 12);
        dht(1, 1, kAcChrBits, kAcChrVals, 162);
    }
    const int mcux = (W + 8 * hs - 1) / (8 * hs), mcuy = (H + 8 * vs - 1) / (8 * vs);
    if (rst) {
        o.insert(o.end(), {0xFF, 0xDD, 0x00, 0x04});
        put16(o, mcux);
    }
    if (grey)
        o.insert(o.end(), {0xFF, 0xDA, 0x00, 0x08, 0x01, 0x01, 0x00, 0x00, 0x3F, 0x00});
    else
        o.insert(o.end(), {0xFF, 0xDA, 0x00, 0x0C, 0x03, 0x01, 0x00, 0x02, 0x11, 0x03, 0x11, 0x00, 0x3F, 0x00});
    // colour planes at full resolution, edges replicated to whole MCUs
    const int PW = mcux * 8 * hs, PH = mcuy * 8 * vs;
    std::vector<float> Y(static_cast<size_t>(PW) * PH), Cb(Y.size()), Cr(Y.size());
    for (int y = 0; y < PH; ++y)
        for (int x = 0; x < PW; ++x) {
            const uint8_t* p = &rgba[(static_cast<size_t>(std::min(y, H - 1)) * W + std::min(x, W - 1)) * 4];
            const float r = p[0], g = p[1], b = p[2];
            const size_t i = static_cast<size_t>(y) * PW + x;
            Y[i] = 0.299f * r + 0.587f * g + 0.114f * b;
            Cb[i] = -0.168736f * r - 0.331264f * g + 0.5f * b + 128.0f;
            Cr[i] = 0.5f * r - 0.418688f * g - 0.081312f * b + 128.0f;
        }
    BitWriter bw(o);
    int pred[3] = {0, 0, 0};
    float blk[64];
    for (int my = 0; my < mcuy; ++my) {
        for (int mx = 0; mx < mcux; ++mx) {
            for (int by = 0; by < vs; ++by)
                for (int bx = 0; bx < hs; ++bx) {
                    const int x0 = (mx * hs + bx) * 8, y0 = (my * vs + by) * 8;
                    for (int j = 0; j < 64; ++j)
                        blk[j] = Y[static_cast<size_t>(y0 + j / 8) * PW + x0 + j % 8] - 128.0f;
                    encode_block(bw, blk, q[0], dcl, acl, &pred[0]);
                }
            for (int c = 0; c < (grey ? 0 : 2); ++c) {
                const std::vector<float>& P = c ? Cr : Cb;
                for (int j = 0; j < 64; ++j) {  // the mean of the hs x vs full-resolution samples
                    float s = 0.0f;
                    for (int dy = 0; dy < vs; ++dy)
                        for (int dx = 0; dx < hs; ++dx)
                            s += P[static_cast<size_t>(my * 8 * vs + (j / 8) * vs + dy) * PW + mx * 8 * hs +
                                   (j % 8) * hs + dx];
                    blk[j] = s / static_cast<float>(hs * vs) - 128.0f;
                }
                encode_block(bw, blk, q[1], dcc, acc, &pred[1 + c]);
            }
        }
        if (rst && my + 1 < mcuy) {
            bw.flush();
            o.push_back(0xFF);
            o.push_back(static_cast<uint8_t>(0xD0 | (my & 7)));
            pred[0] = pred[1] = pred[2] = 0;
        }
    }
    bw.flush();
    o.push_back(0xFF);
    o.push_back(0xD9);
    return VSC_OK;
}

}  // namespace vsc
