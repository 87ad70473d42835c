// Windows BMP and binary PGM / PPM (P5 / P6) decoding, to RGBA bytes, as
// stb_image v2.30 decodes them for `image_texture` (texture.h:78 calls
// stbi_load(path, &w, &h, &channels, 4)).
//
// BMP: info headers of 12 (OS/2), 40, 56, 108 (v4) and 124 (v5) bytes;
// 1, 4 and 8 bits per pixel through a palette, 16 and 32 bits through
// channel masks (5-5-5 and 8-8-8-8 by default, BI_BITFIELDS explicit), 24
// bits as BGR. RLE and embedded JPEG / PNG are not read (stb reads neither).
// The channel count is 4 when the header gives an alpha mask (except a
// 24-bit file whose mask is the default 0xff000000), else 3; a 32-bit
// image whose alpha bytes are all 0 reads as opaque. A field narrower than
// 8 bits widens by bit replication (5-bit abcde -> abcdeabc), which is what
// stb's multiply-and-shift tables compute. Where stb's arithmetic has
// quirks the decoder follows them, because the aim is the same texels:
//  * an OS/2 (12-byte) header's palette holds (offset - 38) / 3 entries;
//  * for 16 to 32 bits, pixel data starts at offset + (offset - end of the
//    header): stb skips the gap after the header twice.
// Palette entries past the stored ones read as black (stb reads
// uninitialised memory there). A file that ends before its pixels do is an
// error here; stb reads zeros past the end.
//
// PNM: P5 (grey, 1 channel) and P6 (RGB, 3 channels), comments and any
// whitespace in the header, data after exactly one byte past the maximum
// value. A maximum above 255 means 16-bit samples; stb_image reduces them to
// 8 bits by keeping the high byte of each sample read as a little-endian
// 16-bit number, i.e. the second byte of the big-endian sample on the
// little-endian machines this runs on, and so does this decoder. A maximum
// below 255 is not rescaled (neither format is).

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "image_reader.h"

namespace mypbr_host {

namespace {

uint32_t le16(const uint8_t* p) { return uint32_t(p[0]) | uint32_t(p[1]) << 8; }
uint32_t le32(const uint8_t* p) {
    return uint32_t(p[0]) | uint32_t(p[1]) << 8 | uint32_t(p[2]) << 16 | uint32_t(p[3]) << 24;
}

int highest_bit(uint32_t v) {
    int n = -1;
    while (v) {
        v >>= 1;
        n++;
    }
    return n;
}

int bit_count(uint32_t v) {
    int n = 0;
    for (; v; v &= v - 1)
        n++;
    return n;
}

// The field `mask` of `v` as 8 bits: the top `bits` bits of the 8-bit window
// ending at the mask's highest bit, repeated downwards to fill the byte.
uint8_t widen_field(uint32_t v, uint32_t mask, int bits) {
    int shift = highest_bit(mask) - 7;
    uint32_t w = v & mask;
    w = shift < 0 ? w << -shift : w >> shift;
    uint32_t top = (w & 0xff) >> (8 - bits);
    uint32_t r = top << (8 - bits);
    for (int s = bits; s < 8; s += bits)
        r |= (top << (8 - bits)) >> s;
    return uint8_t(r);
}

}  // namespace

bool decode_bmp(const uint8_t* b, size_t n, LdrImage& out, std::string& error) {
    error = "not a readable BMP image";
    if (n < 26 || b[0] != 'B' || b[1] != 'M')
        return false;
    const int64_t offset = int32_t(le32(b + 10));
    const uint32_t hsz = le32(b + 14);
    if (offset < 0)
        return false;
    if (hsz != 12 && hsz != 40 && hsz != 56 && hsz != 108 && hsz != 124) {
        error = "BMP header of " + std::to_string(hsz) + " bytes is not supported";
        out.unsupported = true;
        return false;
    }
    size_t header_end = 14 + size_t(hsz);
    if (n < header_end) {
        error = "truncated BMP header";
        return false;
    }
    const uint8_t* h = b + 18;
    int64_t width, height;
    int bpp;
    if (hsz == 12) {
        width = le16(h);
        height = le16(h + 2);
        if (le16(h + 4) != 1)
            return false;
        bpp = int(le16(h + 6));
    } else {
        width = int32_t(le32(h));
        height = int32_t(le32(h + 4));
        if (le16(h + 8) != 1)
            return false;
        bpp = int(le16(h + 10));
    }
    uint32_t mr = 0, mg = 0, mb = 0, ma = 0;
    bool alpha_all_zero_fix = false;  // a default 32-bit alpha channel that may be all 0
    auto default_masks = [&]() {
        if (bpp == 16) {
            mr = 31u << 10;
            mg = 31u << 5;
            mb = 31u;
        } else if (bpp == 32) {
            mr = 0xffu << 16;
            mg = 0xffu << 8;
            mb = 0xffu;
            ma = 0xffu << 24;
            alpha_all_zero_fix = true;
        } else {
            mr = mg = mb = ma = 0;
        }
    };
    if (hsz != 12) {
        uint32_t compress = le32(h + 12);
        if (compress == 1 || compress == 2) {
            error = "run-length encoded BMP images are not supported";
            out.unsupported = true;
            return false;
        }
        if (compress >= 4) {
            error = "BMP images with embedded JPEG or PNG data are not supported";
            out.unsupported = true;
            return false;
        }
        if (compress == 3 && bpp != 16 && bpp != 32)
            return false;
        if (hsz == 40 || hsz == 56) {
            if (bpp == 16 || bpp == 32) {
                if (compress == 0) {
                    default_masks();
                } else {  // compress == 3: the three masks follow the header
                    if (n < header_end + 12) {
                        error = "truncated BMP header";
                        return false;
                    }
                    mr = le32(b + header_end);
                    mg = le32(b + header_end + 4);
                    mb = le32(b + header_end + 8);
                    header_end += 12;
                    if (mr == mg && mg == mb)
                        return false;
                }
            }
        } else {  // v4 / v5: masks in the header
            mr = le32(h + 36);
            mg = le32(h + 40);
            mb = le32(h + 44);
            ma = le32(h + 48);
            if (compress != 3)
                default_masks();
        }
    }
    const bool flip = height > 0;
    if (height < 0)
        height = -height;
    if (width <= 0 || height <= 0 || width > (1 << 15) || height > (1 << 15)) {
        error = "BMP image of " + std::to_string(width) + "x" + std::to_string(height) + " is not supported";
        return false;
    }
    // palette size, as stb computes it
    int64_t psize = 0;
    if (hsz == 12) {
        if (bpp < 24)
            psize = (offset - 14 - 24) / 3;
    } else if (bpp < 16) {
        psize = (offset - int64_t(header_end)) >> 2;
    }
    size_t pos = header_end;
    if (psize == 0) {
        if (offset < int64_t(header_end) || offset - int64_t(header_end) > 1024) {
            error = "BMP pixel offset is outside the file's header";
            return false;
        }
        pos = size_t(offset);
    }
    const int channels = (bpp == 24 && ma == 0xff000000u) ? 3 : (ma ? 4 : 3);
    const size_t w = size_t(width), hh = size_t(height);
    std::vector<uint8_t> px(w * hh * 4);
    auto need = [&](size_t bytes) {
        if (pos + bytes > n) {
            error = "truncated BMP pixel data";
            return false;
        }
        return true;
    };
    if (bpp < 16) {
        if (psize <= 0 || psize > 256) {
            error = "BMP palette of " + std::to_string(psize) + " entries";
            return false;
        }
        if (bpp != 1 && bpp != 4 && bpp != 8) {
            error = "BMP images of " + std::to_string(bpp) + " bits per pixel are not supported";
            out.unsupported = true;
            return false;
        }
        const size_t entry = hsz == 12 ? 3 : 4;
        uint8_t pal[256][3] = {};
        if (!need(size_t(psize) * entry))
            return false;
        for (int64_t i = 0; i < psize; i++) {
            pal[i][0] = b[pos + 2];
            pal[i][1] = b[pos + 1];
            pal[i][2] = b[pos];
            pos += entry;
        }
        pos = size_t(offset);  // header end + palette + any gap
        const size_t row = bpp == 1 ? (w + 7) / 8 : bpp == 4 ? (w + 1) / 2 : w;
        const size_t stride = (row + 3) & ~size_t(3);
        for (size_t y = 0; y < hh; y++) {
            if (!need(row))
                return false;
            const uint8_t* r = b + pos;
            uint8_t* o = &px[(flip ? hh - 1 - y : y) * w * 4];
            for (size_t x = 0; x < w; x++) {
                int v = bpp == 1 ? (r[x >> 3] >> (7 - (x & 7))) & 1 : bpp == 4 ? (r[x >> 1] >> (x & 1 ? 0 : 4)) & 15 : r[x];
                o[4 * x] = pal[v][0];
                o[4 * x + 1] = pal[v][1];
                o[4 * x + 2] = pal[v][2];
                o[4 * x + 3] = 255;
            }
            pos += std::min(stride, n - pos);
        }
    } else {
        pos += size_t(offset) - std::min(size_t(offset), header_end);
        const bool bgr24 = bpp == 24;
        const bool bgra32 = bpp == 32 && mb == 0xffu && mg == 0xff00u && mr == 0xff0000u && ma == 0xff000000u;
        int rc = 0, gc = 0, bc = 0, ac = 0;
        if (!bgr24 && !bgra32) {
            if (!mr || !mg || !mb || (bpp != 16 && bpp != 32)) {
                error = "BMP channel masks are not usable";
                return false;
            }
            rc = bit_count(mr);
            gc = bit_count(mg);
            bc = bit_count(mb);
            ac = bit_count(ma);
            if (rc > 8 || gc > 8 || bc > 8 || ac > 8) {
                error = "BMP channel masks wider than 8 bits are not supported";
                out.unsupported = true;
                return false;
            }
        }
        const size_t bytes = size_t(bpp / 8);
        const size_t row = w * bytes;
        const size_t stride = (row + 3) & ~size_t(3);
        bool any_alpha = false;
        for (size_t y = 0; y < hh; y++) {
            if (!need(row))
                return false;
            const uint8_t* r = b + pos;
            uint8_t* o = &px[(flip ? hh - 1 - y : y) * w * 4];
            for (size_t x = 0; x < w; x++, r += bytes, o += 4) {
                if (bgr24 || bgra32) {
                    o[0] = r[2];
                    o[1] = r[1];
                    o[2] = r[0];
                    o[3] = bgra32 ? r[3] : 255;
                } else {
                    uint32_t v = bpp == 16 ? le16(r) : le32(r);
                    o[0] = widen_field(v, mr, rc);
                    o[1] = widen_field(v, mg, gc);
                    o[2] = widen_field(v, mb, bc);
                    o[3] = ma ? widen_field(v, ma, ac) : 255;
                }
                any_alpha |= o[3] != 0;
            }
            pos += std::min(stride, n - pos);
        }
        if (alpha_all_zero_fix && !any_alpha)
            for (size_t k = 0; k < w * hh; k++)
                px[4 * k + 3] = 255;
    }
    out.width = int(width);
    out.height = int(height);
    out.channels = channels;
    out.rgba = std::move(px);
    error.clear();
    return true;
}

bool decode_pnm(const uint8_t* b, size_t n, LdrImage& out, std::string& error) {
    error = "not a readable PGM / PPM image";
    if (n < 2 || b[0] != 'P' || (b[1] != '5' && b[1] != '6'))
        return false;
    const int channels = b[1] == '6' ? 3 : 1;
    size_t pos = 2;
    // stb's reader: one byte of look-ahead `c`, 0 once the file has ended
    auto next = [&]() -> int { return pos < n ? b[pos++] : 0; };
    auto at_end = [&]() { return pos >= n; };
    int c = next();
    auto space = [](int ch) { return ch == ' ' || ch == '\t' || ch == '\n' || ch == '\v' || ch == '\f' || ch == '\r'; };
    auto skip_space = [&]() {
        for (;;) {
            while (!at_end() && space(c))
                c = next();
            if (at_end() || c != '#')
                break;
            while (!at_end() && c != '\n' && c != '\r')
                c = next();
        }
    };
    bool overflow = false;
    auto integer = [&]() {
        int64_t v = 0;
        while (!at_end() && c >= '0' && c <= '9') {
            v = v * 10 + (c - '0');
            c = next();
            if (v > 214748364 || (v == 214748364 && c > '7')) {
                overflow = true;
                return int64_t(0);
            }
        }
        return v;
    };
    skip_space();
    const int64_t w = integer();
    if (overflow || w == 0) {
        error = "PGM / PPM header has a zero or overflowing width";
        return false;
    }
    skip_space();
    const int64_t h = integer();
    if (overflow || h == 0) {
        error = "PGM / PPM header has a zero or overflowing height";
        return false;
    }
    skip_space();
    const int64_t maxv = integer();
    if (overflow || maxv > 65535) {
        error = "PGM / PPM maximum value above 65535";
        return false;
    }
    if (w > (1 << 15) || h > (1 << 15)) {
        error = "PGM / PPM image of " + std::to_string(w) + "x" + std::to_string(h) + " is not supported";
        return false;
    }
    const size_t sample = maxv > 255 ? 2 : 1;
    const size_t count = size_t(w) * size_t(h);
    const size_t data = count * size_t(channels) * sample;
    if (pos > n || n - pos < data) {
        error = "PGM / PPM file truncated";
        return false;
    }
    const uint8_t* p = b + pos + (sample == 2 ? 1 : 0);
    std::vector<uint8_t> px(count * 4);
    for (size_t k = 0; k < count; k++) {
        uint8_t* o = &px[4 * k];
        if (channels == 1) {
            o[0] = o[1] = o[2] = p[k * sample];
        } else {
            o[0] = p[(3 * k) * sample];
            o[1] = p[(3 * k + 1) * sample];
            o[2] = p[(3 * k + 2) * sample];
        }
        o[3] = 255;
    }
    out.width = int(w);
    out.height = int(h);
    out.channels = channels;
    out.rgba = std::move(px);
    error.clear();
    return true;
}

}  // namespace mypbr_host
