// Decoding of 8-bit image textures (the reference reads them with stb_image,
// texture.h:67-98): RGBA8 out, whatever the file's color type and depth.
//
// PNG first, then TGA further down.
//
// The format (ISO/IEC 15948): a signature, then chunks (length, type, data,
// CRC). IHDR gives size, bit depth, color type and interlacing; PLTE the
// palette; tRNS palette alphas or a transparent grey / RGB key; the IDAT chunks
// together are one zlib stream (RFC 1950) of deflate data (RFC 1951) holding
// the scanlines, each led by a filter byte (none, sub, up, average, Paeth).
// Interlaced images hold seven reduced passes (Adam7). 16-bit samples keep
// their high byte; grey samples below 8 bits are scaled to 0..255.
#include "image_reader.h"

#include <cstring>
#include <fstream>

namespace mypbr_host {

namespace {

// ---------------------------------------------------------------- inflate

struct BitIn {
    const uint8_t* p;
    size_t n, pos = 0;  // pos in bits
    bool bad = false;
    int bit() {
        if ((pos >> 3) >= n) {
            bad = true;
            return 0;
        }
        int b = (p[pos >> 3] >> (pos & 7)) & 1;
        pos++;
        return b;
    }
    uint32_t bits(int k) {  // LSB first
        uint32_t v = 0;
        for (int i = 0; i < k; i++)
            v |= uint32_t(bit()) << i;
        return v;
    }
};

// A canonical Huffman code from code lengths: symbols sorted by (length, value).
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof count);
        for (int i = 0; i < n; i++)
            count[lengths[i]]++;
        count[0] = 0;
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++)
            offs[l + 1] = uint16_t(offs[l] + count[l]);
        symbol.assign(size_t(n), 0);
        for (int i = 0; i < n; i++)
            if (lengths[i])
                symbol[offs[lengths[i]]++] = uint16_t(i);
        return true;
    }
    // Decodes one symbol, reading code bits most significant first.
    int decode(BitIn& in) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= in.bit();
            int c = count[len];
            if (code - first < c)
                return symbol[size_t(index + code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        in.bad = true;
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(BitIn& in, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit) {
    while (!in.bad) {
        int s = lit.decode(in);
        if (s < 0)
            return false;
        if (s < 256) {
            out.push_back(uint8_t(s));
        } else if (s == 256) {
            return true;
        } else {
            s -= 257;
            if (s >= 29)
                return false;
            size_t len = kLenBase[s] + in.bits(kLenExtra[s]);
            int ds = dist.decode(in);
            if (ds < 0 || ds >= 30)
                return false;
            size_t d = kDistBase[ds] + in.bits(kDistExtra[ds]);
            if (d > out.size())
                return false;
            size_t from = out.size() - d;
            for (size_t k = 0; k < len; k++)
                out.push_back(out[from + k]);
        }
        if (out.size() > limit)
            return false;
    }
    return false;
}

// A zlib stream into out (at most `limit` bytes).
bool zlib_inflate(const std::vector<uint8_t>& z, std::vector<uint8_t>& out, size_t limit) {
    if (z.size() < 2 || (z[0] & 15) != 8 || ((z[0] << 8) | z[1]) % 31 != 0 || (z[1] & 32))
        return false;
    BitIn in{z.data() + 2, z.size() - 2};
    bool last = false;
    while (!last) {
        last = in.bit();
        int type = int(in.bits(2));
        if (in.bad)
            return false;
        if (type == 0) {  // stored
            in.pos = (in.pos + 7) & ~size_t(7);
            size_t at = in.pos >> 3;
            if (at + 4 > in.n)
                return false;
            size_t len = in.p[at] | (in.p[at + 1] << 8);
            size_t nlen = in.p[at + 2] | (in.p[at + 3] << 8);
            if ((len ^ 0xffff) != nlen || at + 4 + len > in.n)
                return false;
            out.insert(out.end(), in.p + at + 4, in.p + at + 4 + len);
            in.pos = (at + 4 + len) << 3;
        } else if (type == 1) {  // fixed codes
            uint8_t l[288], d[30];
            for (int i = 0; i < 288; i++)
                l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
            for (int i = 0; i < 30; i++)
                d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            if (!inflate_block(in, lit, dist, out, limit))
                return false;
        } else if (type == 2) {  // dynamic codes
            int hlit = int(in.bits(5)) + 257, hdist = int(in.bits(5)) + 1, hclen = int(in.bits(4)) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; i++)
                cl[order[i]] = uint8_t(in.bits(3));
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[320] = {};
            int k = 0;
            while (k < hlit + hdist && !in.bad) {
                int s = clh.decode(in);
                if (s < 0)
                    return false;
                if (s < 16) {
                    lens[k++] = uint8_t(s);
                } else {
                    int rep = 0, val = 0;
                    if (s == 16) {
                        if (k == 0)
                            return false;
                        val = lens[k - 1];
                        rep = 3 + int(in.bits(2));
                    } else if (s == 17) {
                        rep = 3 + int(in.bits(3));
                    } else {
                        rep = 11 + int(in.bits(7));
                    }
                    if (k + rep > hlit + hdist)
                        return false;
                    while (rep--)
                        lens[k++] = uint8_t(val);
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            if (!inflate_block(in, lit, dist, out, limit))
                return false;
        } else {
            return false;
        }
        if (in.bad)
            return false;
    }
    return true;
}

// ---------------------------------------------------------------- PNG

uint32_t be32(const uint8_t* p) { return uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3]; }

int paeth(int a, int b, int c) {
    int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc)
        return a;
    return pb <= pc ? b : c;
}

// Undoes the scanline filters of a w x h (sub)image in place; returns false
// on an unknown filter. Rows are `stride` bytes after their filter byte.
bool unfilter(uint8_t* data, int h, size_t stride, int bpp) {
    uint8_t* prev = nullptr;
    for (int y = 0; y < h; y++) {
        uint8_t* row = data + size_t(y) * (stride + 1);
        int f = row[0];
        uint8_t* r = row + 1;
        for (size_t x = 0; x < stride; x++) {
            int a = x >= size_t(bpp) ? r[x - bpp] : 0;
            int b = prev ? prev[x] : 0;
            int c = prev && x >= size_t(bpp) ? prev[x - bpp] : 0;
            int v = r[x];
            switch (f) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: return false;
            }
            r[x] = uint8_t(v);
        }
        prev = r;
    }
    return true;
}

}  // namespace

bool read_file_bytes(const std::string& path, std::vector<uint8_t>& bytes) {
    std::ifstream file(path, std::ios::binary);
    if (!file)
        return false;
    bytes.assign((std::istreambuf_iterator<char>(file)), std::istreambuf_iterator<char>());
    return true;
}

ImageKind sniff_image(const uint8_t* b, size_t n) {
    static const uint8_t png_sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    auto starts = [&](const char* text) {
        size_t k = std::strlen(text);
        return n >= k && std::memcmp(b, text, k) == 0;
    };
    if (n >= 8 && std::memcmp(b, png_sig, 8) == 0)
        return ImageKind::Png;
    if (starts("#?RADIANCE\n") || starts("#?RGBE\n"))
        return ImageKind::Hdr;
    if (n >= 3 && b[0] == 0xff && b[1] == 0xd8 && b[2] == 0xff)
        return ImageKind::Jpeg;
    if (starts("BM"))
        return ImageKind::Bmp;
    if (starts("GIF8"))
        return ImageKind::Gif;
    if (starts("P5") || starts("P6"))
        return ImageKind::Pnm;
    if (starts("8BPS"))
        return ImageKind::Psd;
    if (n >= 92 && std::memcmp(b, "\x53\x80\xf6\x34", 4) == 0 && std::memcmp(b + 88, "PICT", 4) == 0)
        return ImageKind::Pic;
    return ImageKind::Other;
}

bool read_ldr_image(const std::string& path, LdrImage& out, std::string& error) {
    std::vector<uint8_t> bytes;
    if (!read_file_bytes(path, bytes)) {
        error = "cannot open '" + path + "'";
        return false;
    }
    return decode_ldr_image(bytes.data(), bytes.size(), out, error);
}

bool decode_ldr_image(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error) {
    switch (sniff_image(bytes, size)) {
        case ImageKind::Png: return decode_png(bytes, size, out, error);
        case ImageKind::Other: return decode_tga(bytes, size, out, error);
        case ImageKind::Jpeg: return decode_jpeg(bytes, size, out, error);
        case ImageKind::Bmp: return decode_bmp(bytes, size, out, error);
        case ImageKind::Pnm: return decode_pnm(bytes, size, out, error);
        case ImageKind::Gif: return decode_gif(bytes, size, out, error);
        case ImageKind::Psd:
            error = "Photoshop (PSD) images are not decoded by this backend";
            out.unsupported = true;
            return false;
        case ImageKind::Pic:
            error = "Softimage PIC images are not decoded by this backend";
            out.unsupported = true;
            return false;
        case ImageKind::Hdr: error = "a Radiance HDR image is not an 8-bit image"; return false;
    }
    return false;
}

bool decode_png(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    if (size < 8 || std::memcmp(bytes, sig, 8) != 0) {
        error = "not a PNG file";
        return false;
    }
    int w = 0, h = 0, depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette, trns;
    size_t pos = 8;
    bool ended = false;
    while (pos + 12 <= size && !ended) {
        uint32_t len = be32(bytes + pos);
        const uint8_t* type = bytes + pos + 4;
        const uint8_t* data = bytes + pos + 8;
        if (len > size - pos - 12) {
            error = "truncated PNG chunk";
            return false;
        }
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            w = int(be32(data));
            h = int(be32(data + 4));
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
        } else if (!std::memcmp(type, "PLTE", 4)) {
            palette.assign(data, data + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(data, data + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            ended = true;
        }
        pos += 12 + len;
    }
    int channels = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
    bool depth_ok = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
    if (w <= 0 || h <= 0 || w > (1 << 15) || h > (1 << 15) || channels == 0 || !depth_ok || interlace > 1 ||
        (ctype == 3 && palette.size() < 3)) {
        error = "unsupported or malformed PNG header";
        return false;
    }
    const int bits_pp = channels * depth;
    const int bpp = std::max(1, bits_pp / 8);
    // passes: the whole image, or Adam7's seven
    struct Pass {
        int x0, y0, dx, dy;
    };
    const Pass adam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                           {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    const Pass whole[1] = {{0, 0, 1, 1}};
    const Pass* passes = interlace ? adam7 : whole;
    int npass = interlace ? 7 : 1;
    size_t expect = 0;
    for (int p = 0; p < npass; p++) {
        size_t pw = size_t((w - passes[p].x0 + passes[p].dx - 1) / passes[p].dx);
        size_t ph = size_t((h - passes[p].y0 + passes[p].dy - 1) / passes[p].dy);
        if (pw && ph)
            expect += ph * (1 + (pw * size_t(bits_pp) + 7) / 8);
    }
    std::vector<uint8_t> raw;
    raw.reserve(expect);
    if (!zlib_inflate(idat, raw, expect + 1024) || raw.size() < expect) {
        error = "corrupt PNG image data";
        return false;
    }
    out.width = w;
    out.height = h;
    out.rgba.assign(size_t(w) * h * 4, 255);
    bool key = !trns.empty() && (ctype == 0 || ctype == 2);
    int key_v[3] = {0, 0, 0};
    if (key && ctype == 0 && trns.size() >= 2)
        key_v[0] = (trns[0] << 8) | trns[1];
    if (key && ctype == 2 && trns.size() >= 6)
        for (int c = 0; c < 3; c++)
            key_v[c] = (trns[2 * c] << 8) | trns[2 * c + 1];
    size_t off = 0;
    for (int p = 0; p < npass; p++) {
        int pw = (w - passes[p].x0 + passes[p].dx - 1) / passes[p].dx;
        int ph = (h - passes[p].y0 + passes[p].dy - 1) / passes[p].dy;
        if (pw <= 0 || ph <= 0)
            continue;
        size_t stride = (size_t(pw) * size_t(bits_pp) + 7) / 8;
        uint8_t* sub = raw.data() + off;
        if (!unfilter(sub, ph, stride, bpp)) {
            error = "corrupt PNG filter";
            return false;
        }
        for (int y = 0; y < ph; y++) {
            const uint8_t* r = sub + size_t(y) * (stride + 1) + 1;
            for (int x = 0; x < pw; x++) {
                int samp[4] = {0, 0, 0, 255};
                int raw_s[4] = {0, 0, 0, 0};  // samples at full depth, for the tRNS key
                for (int c = 0; c < channels; c++) {
                    int v;
                    if (depth == 16) {
                        v = (r[(size_t(x) * channels + c) * 2] << 8) | r[(size_t(x) * channels + c) * 2 + 1];
                        raw_s[c] = v;
                        v >>= 8;
                    } else if (depth == 8) {
                        v = r[size_t(x) * channels + c];
                        raw_s[c] = v;
                    } else {
                        size_t bit = size_t(x) * depth;
                        v = (r[bit >> 3] >> (8 - depth - int(bit & 7))) & ((1 << depth) - 1);
                        raw_s[c] = v;
                        if (ctype == 0)
                            v = v * 255 / ((1 << depth) - 1);
                    }
                    samp[c] = v;
                }
                uint8_t* o = &out.rgba[(size_t(passes[p].y0 + y * passes[p].dy) * w + size_t(passes[p].x0 + x * passes[p].dx)) * 4];
                if (ctype == 3) {
                    size_t i = size_t(samp[0]);
                    if (3 * i + 2 < palette.size()) {
                        o[0] = palette[3 * i];
                        o[1] = palette[3 * i + 1];
                        o[2] = palette[3 * i + 2];
                    } else {
                        o[0] = o[1] = o[2] = 0;
                    }
                    o[3] = i < trns.size() ? trns[i] : 255;
                } else if (ctype == 0 || ctype == 4) {
                    o[0] = o[1] = o[2] = uint8_t(samp[0]);
                    o[3] = ctype == 4 ? uint8_t(samp[1]) : 255;
                    if (key && raw_s[0] == key_v[0])
                        o[3] = 0;
                } else {
                    o[0] = uint8_t(samp[0]);
                    o[1] = uint8_t(samp[1]);
                    o[2] = uint8_t(samp[2]);
                    o[3] = ctype == 6 ? uint8_t(samp[3]) : 255;
                    if (key && raw_s[0] == key_v[0] && raw_s[1] == key_v[1] && raw_s[2] == key_v[2])
                        o[3] = 0;
                }
            }
        }
        off += size_t(ph) * (stride + 1);
    }
    // channels as stb_image reports them: a tRNS chunk adds an alpha channel
    if (ctype == 3)
        out.channels = trns.empty() ? 3 : 4;
    else
        out.channels = channels + (key ? 1 : 0);
    return true;
}

// ---------------------------------------------------------------- TGA
//
// Truevision TGA: an 18-byte header (id length, color-map type, image type,
// color-map start / length / entry bits, origin, width, height, pixel bits,
// descriptor), the id, the color map, then pixels, bottom row first unless
// descriptor bit 5 is set, either plain or run-length coded (type + 8: a
// packet byte whose top bit marks a run of one repeated pixel, low 7 bits the
// count - 1). Types 1 (color-mapped), 2 (true color, BGR[A] or 15/16-bit
// 5:5:5) and 3 (grey). Channels as stb_image counts them: 8-bit grey 1,
// 16-bit grey 2, 15/16-bit color 3 (its top bit is not alpha), 24 3, 32 4.
bool decode_tga(const uint8_t* b, size_t n, LdrImage& out, std::string& error) {
    error = "not a readable TGA image";
    if (n < 18)
        return false;
    int id_len = b[0], map_type = b[1], type = b[2];
    int map_first = b[3] | b[4] << 8, map_len = b[5] | b[6] << 8, map_bits = b[7];
    int w = b[12] | b[13] << 8, h = b[14] | b[15] << 8, bits = b[16], desc = b[17];
    bool rle = type >= 8;
    int base = rle ? type - 8 : type;
    if (map_type > 1 || (base != 1 && base != 2 && base != 3) || w <= 0 || h <= 0 || w > (1 << 15) || h > (1 << 15))
        return false;
    bool mapped = base == 1, grey = base == 3;
    if (mapped && (map_type != 1 || bits != 8 || map_len <= 0))
        return false;
    int pix_bits = mapped ? map_bits : bits;
    int comp;
    bool rgb16 = false;
    switch (pix_bits) {
        case 8: comp = 1; break;
        case 15: comp = 3; rgb16 = true; break;
        case 16:
            if (grey && !mapped) {
                comp = 2;
            } else {
                comp = 3;
                rgb16 = true;
            }
            break;
        case 24: comp = 3; break;
        case 32: comp = 4; break;
        default: return false;
    }
    if (grey && bits != 8 && bits != 16)
        return false;
    if (!mapped && !grey && bits == 8)
        return false;
    size_t pos = 18 + size_t(id_len);
    int entry_bytes = (pix_bits + 7) / 8;
    std::vector<uint8_t> map;
    if (map_type == 1) {
        size_t map_size = size_t(map_len) * size_t((map_bits + 7) / 8);
        if (pos + map_size > n)
            return false;
        map.assign(b + pos, b + pos + map_size);
        pos += map_size;
    }
    // one pixel, from its bytes, to RGBA
    auto decode = [&](const uint8_t* p, uint8_t* o) {
        if (rgb16) {
            int v = p[0] | p[1] << 8;
            o[0] = uint8_t(((v >> 10) & 31) * 255 / 31);
            o[1] = uint8_t(((v >> 5) & 31) * 255 / 31);
            o[2] = uint8_t((v & 31) * 255 / 31);
            o[3] = 255;
        } else if (comp == 1) {
            o[0] = o[1] = o[2] = p[0];
            o[3] = 255;
        } else if (comp == 2) {
            o[0] = o[1] = o[2] = p[0];
            o[3] = p[1];
        } else {
            o[0] = p[2];
            o[1] = p[1];
            o[2] = p[0];
            o[3] = comp == 4 ? p[3] : 255;
        }
    };
    const int in_bytes = mapped ? 1 : entry_bytes;
    const size_t count = size_t(w) * size_t(h);
    std::vector<uint8_t> px(count * 4);
    uint8_t cur[4] = {0, 0, 0, 0};
    auto fetch = [&](uint8_t* o) {
        if (pos + size_t(in_bytes) > n)
            return false;
        if (mapped) {
            int idx = b[pos] - map_first;
            if (idx < 0 || idx >= map_len)
                return false;
            decode(map.data() + size_t(idx) * size_t(entry_bytes), o);
        } else {
            decode(b + pos, o);
        }
        pos += size_t(in_bytes);
        return true;
    };
    size_t k = 0;
    while (k < count) {
        if (!rle) {
            if (!fetch(&px[4 * k]))
                return false;
            k++;
            continue;
        }
        if (pos >= n)
            return false;
        int head = b[pos++];
        size_t run = size_t(head & 127) + 1;
        if (run > count - k)
            run = count - k;
        if (head & 128) {
            if (!fetch(cur))
                return false;
            for (size_t r = 0; r < run; r++, k++)
                std::memcpy(&px[4 * k], cur, 4);
        } else {
            for (size_t r = 0; r < run; r++, k++)
                if (!fetch(&px[4 * k]))
                    return false;
        }
    }
    out.width = w;
    out.height = h;
    out.channels = comp;
    out.rgba.resize(count * 4);
    bool top_first = (desc >> 5) & 1;
    for (int y = 0; y < h; y++) {
        int src = top_first ? y : h - 1 - y;
        std::memcpy(&out.rgba[size_t(y) * w * 4], &px[size_t(src) * w * 4], size_t(w) * 4);
    }
    error.clear();
    return true;
}

}  // namespace mypbr_host
