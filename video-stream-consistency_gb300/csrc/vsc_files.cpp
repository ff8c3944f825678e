// Headless frame-directory driver, the equivalent of FileStabilizer
// (src/stabilization/stabilizefiles.cpp:37-149) without Qt, and the file
// formats it needs:
//   * PNG, 8-bit gray / gray+alpha / RGB / RGBA, not interlaced: read with a
//     DEFLATE decoder written here from RFC 1950/1951 (no zlib dependency),
//     written as RGB with stored (uncompressed) DEFLATE blocks;
//   * binary PPM (P6, maxval 255), read and written;
//   * Middlebury .flo (flowIO.cpp:31-107): tag 202021.25, width, height,
//     then interleaved (u, v) floats, little-endian.
//   * baseline JPEG, read and written (vsc_jpeg.cpp).
// The reference reads *.png and *.jpg through Qt and writes JPEG
// (stabilizefiles.cpp:104-106); here the outputs are PNG files by default
// (lossless) or, with jpeg_quality set, .jpg files as the reference writes
// them, named like the reference's (six-digit frame index).
#include <cuda_runtime.h>
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vsc.h"

namespace vsc {
// set_error lives in vsc_api.cpp
vsc_status set_error(vsc_status s, const char* fmt, ...);
void clear_error();
// vsc_jpeg.cpp
vsc_status jpeg_decode(const uint8_t* d, size_t n, const char* path, int* w, int* h, std::vector<uint8_t>* rgba,
    bool header_only);
vsc_status jpeg_encode(const uint8_t* rgba, int w, int h, int quality, int flags, std::vector<uint8_t>* out);
}  // namespace vsc

namespace {

using vsc::set_error;

// ---- DEFLATE (RFC 1951) --------------------------------------------------------
struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool bad = false;
    uint32_t get(int k)
    {
        while (cnt < k) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            buf |= static_cast<uint32_t>(p[pos++]) << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return v;
    }
    void byte_align()  // the bits left are the rest of the current byte
    {
        buf = 0;
        cnt = 0;
    }
};

// Canonical Huffman code: number of codes per length and the symbols in
// code order; decoded one bit at a time (codes are sent MSB first).
struct Huff {
    int count[16] = {};
    std::vector<int> sym;
    bool build(const uint8_t* len, int n)
    {
        std::fill(count, count + 16, 0);
        for (int i = 0; i < n; ++i)
            count[len[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = (left << 1) - count[l];
            if (left < 0)
                return false;  // over-subscribed
        }
        int offs[16] = {};
        for (int l = 1; l < 15; ++l)
            offs[l + 1] = offs[l] + count[l];
        sym.assign(n, 0);
        for (int i = 0; i < n; ++i)
            if (len[i])
                sym[offs[len[i]]++] = i;
        return true;
    }
    int decode(Bits& b) const
    {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= static_cast<int>(b.get(1));
            if (b.bad)
                return -1;
            const int c = count[l];
            if (code - first < c)
                return sym[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115,
    131, 163, 195, 227, 258};
const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537,
    2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13,
    13};

bool inflate_codes(Bits& b, std::vector<uint8_t>& out, const Huff& lit, const Huff& dist)
{
    for (;;) {
        int s = lit.decode(b);
        if (s < 0)
            return false;
        if (s < 256) {
            out.push_back(static_cast<uint8_t>(s));
        } else if (s == 256) {
            return true;
        } else {
            s -= 257;
            if (s >= 29)
                return false;
            const size_t len = kLenBase[s] + b.get(kLenExtra[s]);
            const int d = dist.decode(b);
            if (d < 0 || d >= 30)
                return false;
            const size_t back = kDistBase[d] + b.get(kDistExtra[d]);
            if (b.bad || back > out.size())
                return false;
            const size_t from = out.size() - back;
            for (size_t i = 0; i < len; ++i)  // may overlap its own output
                out.push_back(out[from + i]);
        }
    }
}

bool inflate(const uint8_t* src, size_t n, std::vector<uint8_t>& out)
{
    Bits b{src, n};
    int last = 0;
    while (!last) {
        last = static_cast<int>(b.get(1));
        const int type = static_cast<int>(b.get(2));
        if (b.bad)
            return false;
        if (type == 0) {
            b.byte_align();
            if (b.pos + 4 > n)
                return false;
            const unsigned len = src[b.pos] | (src[b.pos + 1] << 8);
            const unsigned nlen = src[b.pos + 2] | (src[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || b.pos + len > n)
                return false;
            out.insert(out.end(), src + b.pos, src + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            struct Fixed {  // the fixed codes of RFC 1951 section 3.2.6
                Huff lit, dist;
                Fixed()
                {
                    uint8_t l[288];
                    for (int i = 0; i < 288; ++i)
                        l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
                    lit.build(l, 288);
                    uint8_t d[30];
                    std::fill(d, d + 30, 5);
                    dist.build(d, 30);
                }
            };
            static const Fixed fixed;  // initialised once, thread-safe
            if (!inflate_codes(b, out, fixed.lit, fixed.dist))
                return false;
        } else if (type == 2) {
            const int nlit = static_cast<int>(b.get(5)) + 257;
            const int ndist = static_cast<int>(b.get(5)) + 1;
            const int nclen = static_cast<int>(b.get(4)) + 4;
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < nclen; ++i)
                cl[order[i]] = static_cast<uint8_t>(b.get(3));
            Huff clh;
            if (b.bad || nlit > 286 || ndist > 30 || !clh.build(cl, 19))
                return false;
            uint8_t lens[286 + 30] = {};
            int i = 0;
            while (i < nlit + ndist) {
                const int s = clh.decode(b);
                if (s < 0)
                    return false;
                if (s < 16) {
                    lens[i++] = static_cast<uint8_t>(s);
                    continue;
                }
                int rep = 0;
                uint8_t v = 0;
                if (s == 16) {
                    if (i == 0)
                        return false;
                    v = lens[i - 1];
                    rep = 3 + static_cast<int>(b.get(2));
                } else if (s == 17) {
                    rep = 3 + static_cast<int>(b.get(3));
                } else {
                    rep = 11 + static_cast<int>(b.get(7));
                }
                if (b.bad || i + rep > nlit + ndist)
                    return false;
                while (rep--)
                    lens[i++] = v;
            }
            Huff lit, dist;
            if (!lit.build(lens, nlit) || !dist.build(lens + nlit, ndist))
                return false;
            if (!inflate_codes(b, out, lit, dist))
                return false;
        } else {
            return false;
        }
    }
    return true;
}

uint32_t adler32(const uint8_t* p, size_t n)
{
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

// CRC-32 of PNG chunks (reflected polynomial 0xEDB88320)
uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0)
{
    struct Table {
        uint32_t t[256];
        Table()
        {
            for (uint32_t i = 0; i < 256; ++i) {
                uint32_t c = i;
                for (int k = 0; k < 8; ++k)
                    c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
                t[i] = c;
            }
        }
    };
    static const Table table;  // initialised once, thread-safe
    crc = ~crc;
    for (size_t i = 0; i < n; ++i)
        crc = table.t[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

uint32_t be32(const uint8_t* p) { return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | p[3]; }

bool read_file(const char* path, std::vector<uint8_t>& data)
{
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return false;
    data.clear();
    uint8_t buf[1 << 16];
    size_t r;
    while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0)
        data.insert(data.end(), buf, buf + r);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

struct Image {
    int w = 0, h = 0;
    std::vector<uint8_t> rgba;
};

vsc_status decode_png(const std::vector<uint8_t>& d, const char* path, Image* img, bool header_only)
{
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    if (d.size() < 8 || std::memcmp(d.data(), sig, 8) != 0)
        return set_error(VSC_EINVAL, "%s: not a PNG file", path);
    size_t pos = 8;
    int w = 0, h = 0, depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> idat;
    bool have_ihdr = false;
    while (pos + 12 <= d.size()) {
        const uint32_t len = be32(&d[pos]);
        const uint8_t* type = &d[pos + 4];
        if (len > d.size() - pos - 12)
            return set_error(VSC_EINVAL, "%s: truncated PNG chunk", path);
        const uint8_t* body = &d[pos + 8];
        if (crc32(type, len + 4) != be32(body + len))
            return set_error(VSC_EINVAL, "%s: PNG chunk CRC mismatch", path);
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            w = static_cast<int>(be32(body));
            h = static_cast<int>(be32(body + 4));
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            have_ihdr = true;
            if (header_only)
                break;
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + len;
    }
    if (!have_ihdr || w <= 0 || h <= 0 || w > 65535 || h > 65535)
        return set_error(VSC_EINVAL, "%s: missing or invalid PNG header", path);
    img->w = w;
    img->h = h;
    if (header_only)
        return VSC_OK;
    const int ch = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
    if (depth != 8 || ch == 0 || interlace != 0)
        return set_error(VSC_EUNSUPPORTED, "%s: PNG with bit depth %d, colour type %d, interlace %d (8-bit gray/RGB/"
            "RGBA, not interlaced, are supported)", path, depth, ctype, interlace);
    if (idat.size() < 6 || (idat[0] & 0x0F) != 8 || ((idat[0] << 8) | idat[1]) % 31 != 0 || (idat[1] & 0x20))
        return set_error(VSC_EINVAL, "%s: bad zlib header", path);
    std::vector<uint8_t> raw;
    const size_t stride = static_cast<size_t>(w) * ch;
    raw.reserve((stride + 1) * h);
    if (!inflate(idat.data() + 2, idat.size() - 6, raw))
        return set_error(VSC_EINVAL, "%s: corrupt DEFLATE stream", path);
    if (raw.size() < (stride + 1) * h || adler32(raw.data(), raw.size()) != be32(&idat[idat.size() - 4]))
        return set_error(VSC_EINVAL, "%s: image data truncated or checksum mismatch", path);
    // undo the per-row filters (PNG specification, section 9)
    std::vector<uint8_t> pix(stride * h);
    for (int y = 0; y < h; ++y) {
        const uint8_t f = raw[y * (stride + 1)];
        const uint8_t* in = &raw[y * (stride + 1) + 1];
        uint8_t* row = &pix[y * stride];
        const uint8_t* up = y ? &pix[(y - 1) * stride] : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= static_cast<size_t>(ch) ? row[i - ch] : 0;
            const int b = up ? up[i] : 0;
            const int c = (up && i >= static_cast<size_t>(ch)) ? up[i - ch] : 0;
            int v = in[i];
            switch (f) {
            case 0:
                break;
            case 1:
                v += a;
                break;
            case 2:
                v += b;
                break;
            case 3:
                v += (a + b) >> 1;
                break;
            case 4: {
                const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                break;
            }
            default:
                return set_error(VSC_EINVAL, "%s: unknown PNG filter %d", path, f);
            }
            row[i] = static_cast<uint8_t>(v);
        }
    }
    img->rgba.resize(static_cast<size_t>(w) * h * 4);
    for (size_t i = 0; i < static_cast<size_t>(w) * h; ++i) {
        const uint8_t* s = &pix[i * ch];
        uint8_t* o = &img->rgba[i * 4];
        if (ch <= 2) {
            o[0] = o[1] = o[2] = s[0];
            o[3] = ch == 2 ? s[1] : 255;
        } else {
            o[0] = s[0];
            o[1] = s[1];
            o[2] = s[2];
            o[3] = ch == 4 ? s[3] : 255;
        }
    }
    return VSC_OK;
}

// binary PPM: "P6", width, height, maxval (255), whitespace/comments between
vsc_status decode_ppm(const std::vector<uint8_t>& d, const char* path, Image* img, bool header_only)
{
    size_t pos = 2;
    int vals[3] = {};
    for (int k = 0; k < 3; ++k) {
        for (;;) {
            while (pos < d.size() && std::isspace(d[pos]))
                ++pos;
            if (pos < d.size() && d[pos] == '#') {
                while (pos < d.size() && d[pos] != '\n')
                    ++pos;
                continue;
            }
            break;
        }
        long v = 0;
        size_t start = pos;
        while (pos < d.size() && std::isdigit(d[pos]) && v < 1000000)
            v = v * 10 + (d[pos++] - '0');
        if (pos == start)
            return set_error(VSC_EINVAL, "%s: bad PPM header", path);
        vals[k] = static_cast<int>(v);
    }
    ++pos;  // one whitespace byte ends the header
    if (vals[0] <= 0 || vals[1] <= 0 || vals[0] > 65535 || vals[1] > 65535)
        return set_error(VSC_EINVAL, "%s: bad PPM size", path);
    if (vals[2] != 255)
        return set_error(VSC_EUNSUPPORTED, "%s: PPM maxval %d (255 is supported)", path, vals[2]);
    img->w = vals[0];
    img->h = vals[1];
    if (header_only)
        return VSC_OK;
    const size_t n = static_cast<size_t>(img->w) * img->h;
    if (d.size() < pos + 3 * n)
        return set_error(VSC_EINVAL, "%s: PPM data truncated", path);
    img->rgba.resize(4 * n);
    for (size_t i = 0; i < n; ++i) {
        img->rgba[4 * i] = d[pos + 3 * i];
        img->rgba[4 * i + 1] = d[pos + 3 * i + 1];
        img->rgba[4 * i + 2] = d[pos + 3 * i + 2];
        img->rgba[4 * i + 3] = 255;
    }
    return VSC_OK;
}

vsc_status load_image(const char* path, Image* img, bool header_only)
{
    std::vector<uint8_t> d;
    if (!read_file(path, d))
        return set_error(VSC_EINVAL, "%s: cannot read (%s)", path, std::strerror(errno));
    if (d.size() >= 8 && d[0] == 0x89 && d[1] == 'P' && d[2] == 'N' && d[3] == 'G')
        return decode_png(d, path, img, header_only);
    if (d.size() >= 2 && d[0] == 'P' && d[1] == '6')
        return decode_ppm(d, path, img, header_only);
    if (d.size() >= 3 && d[0] == 0xFF && d[1] == 0xD8 && d[2] == 0xFF)
        return vsc::jpeg_decode(d.data(), d.size(), path, &img->w, &img->h, &img->rgba, header_only);
    return set_error(VSC_EINVAL, "%s: unknown image format", path);
}

void put32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back(static_cast<uint8_t>(x >> 24));
    v.push_back(static_cast<uint8_t>(x >> 16));
    v.push_back(static_cast<uint8_t>(x >> 8));
    v.push_back(static_cast<uint8_t>(x));
}

void put_chunk(std::vector<uint8_t>& file, const char* type, const std::vector<uint8_t>& body)
{
    put32(file, static_cast<uint32_t>(body.size()));
    const size_t at = file.size();
    file.insert(file.end(), type, type + 4);
    file.insert(file.end(), body.begin(), body.end());
    put32(file, crc32(&file[at], body.size() + 4));
}

vsc_status write_png_rgb(const char* path, const uint8_t* rgba, int w, int h)
{
    std::vector<uint8_t> raw;
    raw.reserve((static_cast<size_t>(w) * 3 + 1) * h);
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);  // filter: none
        for (int x = 0; x < w; ++x) {
            const uint8_t* p = rgba + (static_cast<size_t>(y) * w + x) * 4;
            raw.insert(raw.end(), p, p + 3);
        }
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    do {  // stored blocks of at most 65535 bytes
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(static_cast<uint8_t>(len));
        z.push_back(static_cast<uint8_t>(len >> 8));
        z.push_back(static_cast<uint8_t>(~len));
        z.push_back(static_cast<uint8_t>(~len >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    put32(z, adler32(raw.data(), raw.size()));
    std::vector<uint8_t> file = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<uint8_t> ihdr;
    put32(ihdr, static_cast<uint32_t>(w));
    put32(ihdr, static_cast<uint32_t>(h));
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});  // 8-bit RGB, deflate, adaptive filtering, no interlace
    put_chunk(file, "IHDR", ihdr);
    put_chunk(file, "IDAT", z);
    put_chunk(file, "IEND", {});
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return set_error(VSC_EINVAL, "%s: cannot write (%s)", path, std::strerror(errno));
    const bool ok = std::fwrite(file.data(), 1, file.size(), f) == file.size();
    if (std::fclose(f) != 0 || !ok)
        return set_error(VSC_EINVAL, "%s: write failed", path);
    return VSC_OK;
}

// ---- .flo (flowIO.cpp:31-107) -----------------------------------------------------
vsc_status write_jpeg_rgb(const char* path, const uint8_t* rgba, int w, int h, int quality, int flags)
{
    std::vector<uint8_t> file;
    vsc_status s = vsc::jpeg_encode(rgba, w, h, quality, flags, &file);
    if (s)
        return s;
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return set_error(VSC_EINVAL, "%s: cannot write (%s)", path, std::strerror(errno));
    const bool ok = std::fwrite(file.data(), 1, file.size(), f) == file.size();
    if (std::fclose(f) != 0 || !ok)
        return set_error(VSC_EINVAL, "%s: write failed", path);
    return VSC_OK;
}

vsc_status flo_read(const char* path, std::vector<float>* flow, int* w, int* h)
{
    std::vector<uint8_t> d;
    if (!read_file(path, d))
        return set_error(VSC_EINVAL, "%s: cannot read (%s)", path, std::strerror(errno));
    if (d.size() < 12)
        return set_error(VSC_EINVAL, "%s: problem reading flow file header", path);
    float tag;
    int32_t ww, hh;
    std::memcpy(&tag, &d[0], 4);
    std::memcpy(&ww, &d[4], 4);
    std::memcpy(&hh, &d[8], 4);
    if (tag != 202021.25f)
        return set_error(VSC_EINVAL, "%s: wrong flow file tag", path);
    if (ww < 1 || ww > 99999 || hh < 1 || hh > 99999)
        return set_error(VSC_EINVAL, "%s: illegal flow size %dx%d", path, ww, hh);
    const size_t n = static_cast<size_t>(ww) * hh * 2;
    if (d.size() != 12 + n * 4)
        return set_error(VSC_EINVAL, "%s: flow file is too %s", path, d.size() < 12 + n * 4 ? "short" : "long");
    *w = ww;
    *h = hh;
    if (flow) {
        flow->resize(n);
        std::memcpy(flow->data(), &d[12], n * 4);
    }
    return VSC_OK;
}

vsc_status flo_write(const char* path, const float* flow, int w, int h)
{
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return set_error(VSC_EINVAL, "%s: cannot write (%s)", path, std::strerror(errno));
    const float tag = 202021.25f;
    const int32_t ww = w, hh = h;
    const size_t n = static_cast<size_t>(w) * h * 2;
    bool ok = std::fwrite(&tag, 4, 1, f) == 1 && std::fwrite(&ww, 4, 1, f) == 1 && std::fwrite(&hh, 4, 1, f) == 1 &&
              std::fwrite(flow, 4, n, f) == n;
    if (std::fclose(f) != 0 || !ok)
        return set_error(VSC_EINVAL, "%s: write failed", path);
    return VSC_OK;
}

// ---- the driver -----------------------------------------------------------------------
bool has_image_ext(const std::string& n)
{
    auto ends = [&](const char* e) {
        const size_t l = std::strlen(e);
        return n.size() > l && n.compare(n.size() - l, l, e) == 0;
    };
    return ends(".png") || ends(".jpg") || ends(".jpeg") || ends(".ppm");
}

vsc_status list_frames(const char* dir, std::vector<std::string>* out)
{
    DIR* d = opendir(dir);
    if (!d)
        return set_error(VSC_EINVAL, "frame directory %s does not exist", dir);
    out->clear();
    while (dirent* e = readdir(d)) {
        std::string n = e->d_name;
        if (has_image_ext(n))
            out->push_back(n);
    }
    closedir(d);
    std::sort(out->begin(), out->end());  // QDir::Name
    for (auto& n : *out)
        n = std::string(dir) + "/" + n;
    return VSC_OK;
}

std::string index6(int i)
{
    char b[32];
    std::snprintf(b, sizeof(b), "%06d", i);
    return b;
}

// QImage::scaled(w, h) with the default fast transformation: the source
// pixel under each target pixel centre.
void resize_nearest_rgba(const Image& in, int w, int h, Image* out)
{
    out->w = w;
    out->h = h;
    out->rgba.resize(static_cast<size_t>(w) * h * 4);
    for (int y = 0; y < h; ++y) {
        const int sy = std::min(in.h - 1, static_cast<int>((2LL * y + 1) * in.h / (2LL * h)));
        for (int x = 0; x < w; ++x) {
            const int sx = std::min(in.w - 1, static_cast<int>((2LL * x + 1) * in.w / (2LL * w)));
            std::memcpy(&out->rgba[(static_cast<size_t>(y) * w + x) * 4],
                &in.rgba[(static_cast<size_t>(sy) * in.w + sx) * 4], 4);
        }
    }
}

vsc_status load_frame_file(const std::string& path, int w, int h, Image* img)
{
    Image raw;
    vsc_status s = load_image(path.c_str(), &raw, false);
    if (s)
        return s;
    if (raw.w == w && raw.h == h) {
        *img = std::move(raw);
        return VSC_OK;
    }
    resize_nearest_rgba(raw, w, h, img);
    return VSC_OK;
}

// The reference writes frames through gpuToImage, i.e. after the float
// conversion and back (gpuimage.cu:39-67); so do the first and last frames here.
vsc_status roundtrip_rgba(const Image& in, std::vector<uint8_t>* out, cudaStream_t st)
{
    const size_t n = static_cast<size_t>(in.w) * in.h;
    uint8_t* d8 = nullptr;
    float* df = nullptr;
    cudaError_t e = cudaMalloc(&d8, n * 4);
    if (e == cudaSuccess)
        e = cudaMalloc(&df, n * 12);
    vsc_status s = VSC_OK;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d8, in.rgba.data(), n * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        vsc_image im{df, in.w, in.h, 3};
        if ((s = vsc_char_to_float_image(d8, &im, st)) == VSC_OK && (s = vsc_float_to_char_image(&im, d8, st)) == VSC_OK) {
            out->resize(n * 4);
            e = cudaMemcpyAsync(out->data(), d8, n * 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
        }
    }
    cudaFree(d8);
    cudaFree(df);
    if (s)
        return s;
    if (e != cudaSuccess)
        return set_error(VSC_ECUDA, "files: %s", cudaGetErrorString(e));
    return VSC_OK;
}

}  // namespace

extern "C" {

VSC_API vsc_status vsc_image_file_info(const char* path, int32_t* width, int32_t* height)
{
    vsc::clear_error();
    if (!path || !width || !height)
        return set_error(VSC_EINVAL, "image_file_info: null argument");
    Image img;
    vsc_status s = load_image(path, &img, true);
    if (s)
        return s;
    *width = img.w;
    *height = img.h;
    return VSC_OK;
}

VSC_API vsc_status vsc_read_image_file(const char* path, uint8_t* rgba, int32_t width, int32_t height)
{
    vsc::clear_error();
    if (!path || !rgba)
        return set_error(VSC_EINVAL, "read_image_file: null argument");
    Image img;
    vsc_status s = load_image(path, &img, false);
    if (s)
        return s;
    if (img.w != width || img.h != height)
        return set_error(VSC_EINVAL, "%s: image is %dx%d, expected %dx%d", path, img.w, img.h, width, height);
    std::memcpy(rgba, img.rgba.data(), img.rgba.size());
    return VSC_OK;
}

VSC_API vsc_status vsc_write_png(const char* path, const uint8_t* rgba, int32_t width, int32_t height)
{
    vsc::clear_error();
    if (!path || !rgba || width <= 0 || height <= 0)
        return set_error(VSC_EINVAL, "write_png: bad argument");
    return write_png_rgb(path, rgba, width, height);
}

VSC_API vsc_status vsc_write_jpeg(const char* path, const uint8_t* rgba, int32_t width, int32_t height,
    int32_t quality, int32_t flags)
{
    vsc::clear_error();
    if (!path || !rgba || width < 1 || height < 1)
        return set_error(VSC_EINVAL, "write_jpeg: null argument or empty image");
    if (flags & ~7)
        return set_error(VSC_EINVAL, "write_jpeg: unknown flags 0x%x", flags);
    return write_jpeg_rgb(path, rgba, width, height, quality, flags);
}

VSC_API vsc_status vsc_flo_info(const char* path, int32_t* width, int32_t* height)
{
    vsc::clear_error();
    if (!path || !width || !height)
        return set_error(VSC_EINVAL, "flo_info: null argument");
    int w = 0, h = 0;
    vsc_status s = flo_read(path, nullptr, &w, &h);
    if (s)
        return s;
    *width = w;
    *height = h;
    return VSC_OK;
}

VSC_API vsc_status vsc_read_flo(const char* path, float* flow, int32_t width, int32_t height)
{
    vsc::clear_error();
    if (!path || !flow)
        return set_error(VSC_EINVAL, "read_flo: null argument");
    std::vector<float> v;
    int w = 0, h = 0;
    vsc_status s = flo_read(path, &v, &w, &h);
    if (s)
        return s;
    if (w != width || h != height)  // initializeFlowImage (imagehelpers.cpp:42-50)
        return set_error(VSC_EINVAL, "%s: flow image size %dx%d does not match image size %dx%d", path, w, h, width,
            height);
    std::memcpy(flow, v.data(), v.size() * 4);
    return VSC_OK;
}

VSC_API vsc_status vsc_write_flo(const char* path, const float* flow, int32_t width, int32_t height)
{
    vsc::clear_error();
    if (!path || !flow || width <= 0 || height <= 0)
        return set_error(VSC_EINVAL, "write_flo: bad argument");
    return flo_write(path, flow, width, height);
}

VSC_API vsc_status vsc_stabilize_files(const vsc_files_config* cfg, int32_t* frames_written)
{
    vsc::clear_error();
    if (!cfg || !cfg->original_dir || !cfg->processed_dir || !cfg->output_dir)
        return set_error(VSC_EINVAL, "stabilize_files: null argument");
    if (frames_written)
        *frames_written = 0;
    std::vector<std::string> orig, proc;
    vsc_status s;
    if ((s = list_frames(cfg->original_dir, &orig)) || (s = list_frames(cfg->processed_dir, &proc)))
        return s;
    if (cfg->flow_dir) {
        struct stat sb;
        if (stat(cfg->flow_dir, &sb) != 0 || !S_ISDIR(sb.st_mode))
            return set_error(VSC_EINVAL, "optical flow directory %s does not exist", cfg->flow_dir);
    }
    const int n = static_cast<int>(std::min(orig.size(), proc.size()));
    if (n < 3)
        return set_error(VSC_EINVAL, "stabilize_files: %d frames, at least 3 are needed", n);
    if (cfg->jpeg_quality < 0 || cfg->jpeg_quality > 100)
        return set_error(VSC_EINVAL, "stabilize_files: jpeg_quality %d outside [0, 100]", cfg->jpeg_quality);
    mkdir(cfg->output_dir, 0755);
    int w = cfg->width, h = cfg->height;
    if (w <= 0 || h <= 0) {
        Image first;
        if ((s = load_image(orig[0].c_str(), &first, true)))
            return s;
        w = first.w;
        h = first.h;
    }
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(VSC_ECUDA, "stabilize_files: stream creation failed");
    vsc_stabilizer_config sc{};
    sc.width = w;
    sc.height = h;
    sc.batch_size = 1;
    sc.compute_flow = cfg->flow_dir ? 0 : 1;
    sc.flow_downscale = cfg->flow_downscale > 0 ? cfg->flow_downscale : 1;
    sc.flow_channels = 2;
    sc.use_graphs = 1;
    sc.corr_dtype = cfg->corr_dtype;
    vsc_stabilizer* stab = nullptr;
    if ((s = vsc_stabilizer_create(&sc, st, &stab))) {
        const std::string msg = vsc_last_error();
        cudaStreamDestroy(st);
        return set_error(s, "%s", msg.c_str());
    }
    if (cfg->hyper)
        *vsc_stabilizer_hyper_params(stab) = *cfg->hyper;
    const std::string out_dir = cfg->output_dir;
    int written = 0;
    std::vector<uint8_t> out(static_cast<size_t>(w) * h * 4), rt;
    std::vector<float> ffwd, fbwd;
    Image window[3];
    const int jq = cfg->jpeg_quality;
    auto write = [&](int idx, const uint8_t* rgba) {
        vsc_status r = jq > 0 ? write_jpeg_rgb((out_dir + "/" + index6(idx) + ".jpg").c_str(), rgba, w, h, jq, 0)
                              : write_png_rgb((out_dir + "/" + index6(idx) + ".png").c_str(), rgba, w, h);
        if (!r)
            ++written;
        return r;
    };
    // preloadProcessedFrames (videostabilizer.cpp:136-153): frames 0..2 in, the
    // first two processed frames out (frame 1 is overwritten by its step)
    for (int j = 0; j < 3 && !s; ++j) {
        Image o;
        if ((s = load_frame_file(orig[j], w, h, &o)) || (s = load_frame_file(proc[j], w, h, &window[j])))
            break;
        s = vsc_stabilizer_load_frame(stab, o.rgba.data(), window[j].rgba.data(), 0);
        if (!s && j <= 1 && !(s = roundtrip_rgba(window[j], &rt, st)))
            s = write(j, rt.data());
    }
    for (int i = 1; !s; ++i) {  // doOneStep(i), videostabilizer.cpp:167-265
        if (cfg->flow_dir) {
            // flow file i+1: i -> i+1; "_bwd" file i: i -> i-1 (stabilizefiles.cpp:134-149)
            const std::string fd = cfg->flow_dir;
            ffwd.resize(static_cast<size_t>(w) * h * 2);
            fbwd.resize(ffwd.size());
            if ((s = vsc_read_flo((fd + "/frame_" + index6(i + 1) + ".flo").c_str(), ffwd.data(), w, h)) ||
                (s = vsc_read_flo((fd + "/frame_" + index6(i) + "_bwd.flo").c_str(), fbwd.data(), w, h)) ||
                (s = vsc_stabilizer_set_flows(stab, ffwd.data(), fbwd.data(), 0)))
                break;
        }
        if ((s = vsc_stabilizer_step(stab, out.data(), 0)) || (s = write(i, out.data())))
            break;
        if (i + 2 >= n) {  // outputFinalFrames: the window's next processed frame
            if (!(s = roundtrip_rgba(window[(i + 1) % 3], &rt, st)))
                s = write(i + 1, rt.data());
            break;
        }
        Image o;
        if ((s = load_frame_file(orig[i + 2], w, h, &o)) || (s = load_frame_file(proc[i + 2], w, h, &window[(i + 2) % 3])))
            break;
        s = vsc_stabilizer_load_frame(stab, o.rgba.data(), window[(i + 2) % 3].rgba.data(), 0);
    }
    const std::string msg = s ? vsc_last_error() : "";  // the clean-up calls reset the message
    vsc_stabilizer_destroy(stab);
    cudaStreamDestroy(st);
    if (frames_written)
        *frames_written = s ? written : n;  // frame 1 is written twice (preload, then its step)
    return s ? set_error(s, "%s", msg.c_str()) : VSC_OK;
}

}  // extern "C"
