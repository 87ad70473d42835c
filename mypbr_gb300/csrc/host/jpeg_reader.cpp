// JPEG decoding (ITU-T T.81, JFIF) for 8-bit image textures, as stb_image
// reads them for the reference (texture.h:67-98): sequential and progressive
// Huffman-coded frames (SOF0 / SOF1 / SOF2) of 1 or 3 components with any
// sampling factors, restart intervals, 8- or 16-bit quantisation tables.
// Progressive scans (T.81 G.1.2) fill quantised coefficients band by band:
// DC first and refinement bits, AC first passes with end-of-band runs, AC
// refinement (correction bits for coefficients already nonzero, new ones of
// magnitude 1 << Al); the frame is transformed once all scans are in.
// Lossless, arithmetic-coded and 12-bit files are reported as unsupported.
//
// Per 8 x 8 block: Huffman-decoded DC difference and run-length AC
// coefficients (zigzag order), dequantised, an inverse DCT evaluated as two
// separable passes of the cosine basis in FP32, +128 and clamped. Chroma
// planes subsampled 2:1 are brought to full size with the triangle filter of
// libjpeg's "fancy" upsampling (3/4 of the nearer sample, 1/4 of the farther;
// both directions for 2 x 2), other factors by repetition; YCbCr to RGB by
// the JFIF equations. The result can differ from stb_image's integer IDCT and
// fixed-point colour conversion by a count or two per channel (both are
// within the standard's accuracy); the tests bound that difference.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "image_reader.h"

namespace mypbr_host {

namespace {

const int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                         41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                         30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct HuffTable {
    bool present = false;
    // canonical code: for each length 1..16, the first code and the index of
    // its first symbol, and the count
    int first_code[17] = {}, first_index[17] = {}, count[17] = {};
    uint8_t symbols[256] = {};
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0;
    int td = 0, ta = 0;  // Huffman tables of the current scan
    int bw = 0, bh = 0;  // blocks across and down, padded to whole MCUs
    std::vector<uint8_t> plane;  // bw * 8 x bh * 8 samples
    std::vector<int16_t> coef;   // progressive frames: quantised coefficients, 64 per block in zigzag order
    int dc = 0;
};

struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t acc = 0;
    int have = 0;
    bool marker = false;  // a marker was met: only zero bits follow
    bool fill() {
        while (have <= 24) {
            uint32_t b = 0;
            if (!marker && pos < n) {
                b = p[pos];
                if (b == 0xff) {
                    uint8_t next = pos + 1 < n ? p[pos + 1] : 0;
                    if (next == 0x00) {
                        pos += 2;
                    } else {
                        marker = true;  // RSTn or the end: do not consume
                        b = 0;
                    }
                } else {
                    pos++;
                }
            }
            acc |= b << (24 - have);
            have += 8;
        }
        return true;
    }
    int bit() {
        if (have < 1)
            fill();
        int b = int(acc >> 31);
        acc <<= 1;
        have--;
        return b;
    }
    int bits(int k) {
        if (k == 0)
            return 0;
        if (have < k)
            fill();
        int v = int(acc >> (32 - k));
        acc <<= k;
        have -= k;
        return v;
    }
    void reset() {  // at a restart marker: drop buffered bits
        acc = 0;
        have = 0;
        marker = false;
    }
};

int decode_symbol(Bits& b, const HuffTable& t) {
    int code = 0;
    for (int len = 1; len <= 16; len++) {
        code = (code << 1) | b.bit();
        if (t.count[len] && code - t.first_code[len] < t.count[len] && code >= t.first_code[len])
            return t.symbols[t.first_index[len] + code - t.first_code[len]];
    }
    return -1;
}

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

uint16_t be16(const uint8_t* p) { return uint16_t(p[0] << 8 | p[1]); }

// the separable inverse DCT's basis: c(u) cos((2x + 1) u pi / 16) / 2
struct Idct {
    float basis[8][8];
    Idct() {
        for (int x = 0; x < 8; x++)
            for (int u = 0; u < 8; u++) {
                double cu = u == 0 ? std::sqrt(0.5) : 1.0;
                basis[x][u] = float(cu * std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16) / 2);
            }
    }
    void run(const int* coef, uint8_t* out, int stride) const {
        float tmp[8][8];
        for (int v = 0; v < 8; v++)  // rows of coefficients -> columns of samples
            for (int x = 0; x < 8; x++) {
                float s = 0;
                for (int u = 0; u < 8; u++)
                    s += basis[x][u] * float(coef[v * 8 + u]);
                tmp[v][x] = s;
            }
        for (int y = 0; y < 8; y++)
            for (int x = 0; x < 8; x++) {
                float s = 0;
                for (int v = 0; v < 8; v++)
                    s += basis[y][v] * tmp[v][x];
                int q = int(std::lround(s + 128.0f));
                out[y * stride + x] = uint8_t(std::clamp(q, 0, 255));
            }
    }
};

// a plane subsampled by (sh, sv) brought to full size w x h
void upsample(const Component& c, int sh, int sv, int w, int h, std::vector<uint8_t>& full) {
    full.assign(size_t(w) * h, 0);
    int pw = c.bw * 8;
    int cw = (w + sh - 1) / sh, ch = (h + sv - 1) / sv;  // the samples that cover the image
    auto at = [&](int x, int y) {
        x = std::clamp(x, 0, cw - 1);
        y = std::clamp(y, 0, ch - 1);
        return int(c.plane[size_t(y) * pw + x]);
    };
    if (sh == 1 && sv == 1) {
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++)
                full[size_t(y) * w + x] = uint8_t(at(x, y));
    } else if (sh == 2 && sv == 1) {
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                int i = x >> 1, near = at(i, y), far = at((x & 1) ? i + 1 : i - 1, y);
                int v = (3 * near + far + ((x & 1) ? 2 : 1)) >> 2;
                // stb_image weighs the last sample's left output the other way
                // round (3 x its left neighbour + itself); the reference's
                // textures hold those bytes
                if (!(x & 1) && cw >= 2 && i == cw - 1)
                    v = (3 * at(i - 1, y) + near + 2) >> 2;
                full[size_t(y) * w + x] = uint8_t(v);
            }
    } else if (sh == 1 && sv == 2) {
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                int j = y >> 1, near = at(x, j), far = at(x, (y & 1) ? j + 1 : j - 1);
                full[size_t(y) * w + x] = uint8_t((3 * near + far + 2) >> 2);
            }
    } else if (sh == 2 && sv == 2) {
        // vertical 3:1 blend at 4x the scale, then horizontal 3:1 with rounding
        for (int y = 0; y < h; y++) {
            int j = y >> 1, j2 = (y & 1) ? j + 1 : j - 1;
            for (int x = 0; x < w; x++) {
                int i = x >> 1, i2 = (x & 1) ? i + 1 : i - 1;
                int col_near = 3 * at(i, j) + at(i, j2);
                int col_far = 3 * at(i2, j) + at(i2, j2);
                full[size_t(y) * w + x] = uint8_t((3 * col_near + col_far + ((x & 1) ? 7 : 8)) >> 4);
            }
        }
    } else {
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++)
                full[size_t(y) * w + x] = uint8_t(at(x / sh, y / sv));
    }
}

}  // namespace

bool decode_jpeg(const uint8_t* b, size_t n, LdrImage& out, std::string& error) {
    if (n < 4 || b[0] != 0xff || b[1] != 0xd8) {
        error = "not a JPEG file";
        return false;
    }
    uint16_t quant[4][64] = {};
    HuffTable dc[4], ac[4];
    std::vector<Component> comps;
    int width = 0, height = 0, hmax = 1, vmax = 1, restart = 0;
    bool frame = false, adobe_rgb = false, adobe = false, progressive = false;
    size_t pos = 2;
    static const Idct idct;
    auto corrupt = [&](const char* what) {
        error = std::string("corrupt JPEG: ") + what;
        return false;
    };
    while (pos + 4 <= n) {
        if (b[pos] != 0xff) {
            pos++;
            continue;
        }
        uint8_t m = b[pos + 1];
        if (m == 0xff) {
            pos++;
            continue;
        }
        if (m == 0xd9)
            break;  // EOI
        if (m == 0xd8 || (m >= 0xd0 && m <= 0xd7) || m == 0x01) {
            pos += 2;
            continue;
        }
        size_t len = be16(b + pos + 2);
        if (len < 2 || pos + 2 + len > n)
            return corrupt("segment past the end");
        const uint8_t* s = b + pos + 4;
        size_t sl = len - 2;
        if (m == 0xdb) {  // DQT
            size_t k = 0;
            while (k < sl) {
                int pq = s[k] >> 4, tq = s[k] & 15;
                k++;
                if (tq > 3 || k + (pq ? 128 : 64) > sl)
                    return corrupt("quantisation table");
                for (int i = 0; i < 64; i++)
                    quant[tq][kZigzag[i]] = pq ? be16(s + k + 2 * i) : s[k + i];
                k += pq ? 128 : 64;
            }
        } else if (m == 0xc4) {  // DHT
            size_t k = 0;
            while (k < sl) {
                if (k + 17 > sl)
                    return corrupt("Huffman table");
                int tc = s[k] >> 4, th = s[k] & 15;
                if (tc > 1 || th > 3)
                    return corrupt("Huffman table class");
                HuffTable& t = tc ? ac[th] : dc[th];
                t = HuffTable();
                int total = 0;
                for (int l = 1; l <= 16; l++) {
                    t.count[l] = s[k + l];
                    total += t.count[l];
                }
                if (total > 256 || k + 17 + size_t(total) > sl)
                    return corrupt("Huffman table size");
                std::memcpy(t.symbols, s + k + 17, size_t(total));
                int code = 0, index = 0;
                for (int l = 1; l <= 16; l++) {
                    t.first_code[l] = code;
                    t.first_index[l] = index;
                    code = (code + t.count[l]) << 1;
                    index += t.count[l];
                }
                t.present = true;
                k += 17 + size_t(total);
            }
        } else if (m == 0xdd) {  // DRI
            if (sl < 2)
                return corrupt("restart interval");
            restart = be16(s);
        } else if (m == 0xee) {  // APP14 Adobe: the colour transform
            if (sl >= 12 && std::memcmp(s, "Adobe", 5) == 0) {
                adobe = true;
                adobe_rgb = s[11] == 0;
            }
        } else if (m == 0xc0 || m == 0xc1 || m == 0xc2) {  // SOF0 / SOF1 / SOF2 (progressive)
            progressive = m == 0xc2;
            if (sl < 6 || s[0] != 8) {
                error = "JPEG images of 12-bit precision are not decoded by this backend";
                out.unsupported = true;
                return false;
            }
            height = be16(s + 1);
            width = be16(s + 3);
            int nc = s[5];
            if (width <= 0 || height <= 0 || width > (1 << 15) || height > (1 << 15) || (nc != 1 && nc != 3) ||
                sl < 6 + 3 * size_t(nc)) {
                error = nc == 4 ? "CMYK JPEG images are not decoded by this backend" : "unsupported JPEG frame";
                return false;
            }
            comps.resize(size_t(nc));
            for (int c = 0; c < nc; c++) {
                comps[size_t(c)].id = s[6 + 3 * c];
                comps[size_t(c)].h = s[7 + 3 * c] >> 4;
                comps[size_t(c)].v = s[7 + 3 * c] & 15;
                comps[size_t(c)].tq = s[8 + 3 * c] & 3;
                if (comps[size_t(c)].h < 1 || comps[size_t(c)].h > 4 || comps[size_t(c)].v < 1 || comps[size_t(c)].v > 4)
                    return corrupt("sampling factors");
                hmax = std::max(hmax, comps[size_t(c)].h);
                vmax = std::max(vmax, comps[size_t(c)].v);
            }
            int mcux = (width + 8 * hmax - 1) / (8 * hmax), mcuy = (height + 8 * vmax - 1) / (8 * vmax);
            for (auto& c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.plane.assign(size_t(c.bw) * 8 * size_t(c.bh) * 8, 0);
                if (progressive)
                    c.coef.assign(size_t(c.bw) * size_t(c.bh) * 64, 0);
            }
            frame = true;
        } else if (m == 0xc3 || (m >= 0xc5 && m <= 0xcf && m != 0xc8 && m != 0xcc)) {
            error = "lossless, hierarchical or arithmetic-coded JPEG images are not decoded by this backend";
            out.unsupported = true;
            return false;
        } else if (m == 0xda) {  // SOS: the (single, interleaved or not) scan
            if (!frame)
                return corrupt("scan before frame");
            int ns = s[0];
            if (ns < 1 || ns > 4 || sl < 1 + 2 * size_t(ns) + 3)
                return corrupt("scan header");
            std::vector<Component*> sc;
            for (int i = 0; i < ns; i++) {
                Component* found = nullptr;
                for (auto& c : comps)
                    if (c.id == s[1 + 2 * i])
                        found = &c;
                if (!found)
                    return corrupt("scan component");
                found->td = s[2 + 2 * i] >> 4;
                found->ta = s[2 + 2 * i] & 15;
                if (found->td > 3 || found->ta > 3)
                    return corrupt("Huffman table index");
                sc.push_back(found);
            }
            // spectral selection and successive approximation (progressive scans)
            int ss = s[1 + 2 * ns], se = s[2 + 2 * ns], ah = s[3 + 2 * ns] >> 4, al = s[3 + 2 * ns] & 15;
            for (auto* c : sc) {
                bool need_dc = progressive ? (ss == 0 && ah == 0) : true;
                bool need_ac = progressive ? ss > 0 : true;
                if ((need_dc && !dc[c->td].present) || (need_ac && !ac[c->ta].present))
                    return corrupt("missing Huffman table");
            }
            if (progressive && (se > 63 || ss > se || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13))
                return corrupt("progressive scan parameters");
            pos += 2 + len;
            Bits bits{b + pos, n - pos};
            int eobrun = 0;
            // one block of a progressive scan, into the component's coefficients
            auto prog_block = [&](Component& c, int bx, int by) {
                if (bx >= c.bw || by >= c.bh)
                    return true;
                int16_t* z = &c.coef[(size_t(by) * c.bw + size_t(bx)) * 64];
                if (ss == 0) {  // DC
                    if (ah == 0) {
                        int t = decode_symbol(bits, dc[c.td]);
                        if (t < 0 || t > 11)
                            return false;
                        c.dc += extend(bits.bits(t), t);
                        z[0] = int16_t(c.dc * (1 << al));
                    } else if (bits.bit()) {
                        z[0] = int16_t(z[0] | (1 << al));
                    }
                    return true;
                }
                if (ah == 0) {  // AC, first pass of this band
                    if (eobrun > 0) {
                        eobrun--;
                        return true;
                    }
                    for (int k = ss; k <= se; k++) {
                        int rs = decode_symbol(bits, ac[c.ta]);
                        if (rs < 0)
                            return false;
                        int r = rs >> 4, sz = rs & 15;
                        if (sz == 0) {
                            if (r < 15) {  // a run of end-of-bands
                                eobrun = (1 << r) - 1 + (r ? bits.bits(r) : 0);
                                break;
                            }
                            k += 15;  // sixteen zeros
                            continue;
                        }
                        k += r;
                        if (k > se)
                            return false;
                        z[k] = int16_t(extend(bits.bits(sz), sz) * (1 << al));
                    }
                    return true;
                }
                // AC refinement: a correction bit for every coefficient already
                // nonzero, new coefficients of magnitude 1 << al
                int p1 = 1 << al, m1 = -(1 << al);
                int k = ss;
                if (eobrun == 0) {
                    for (; k <= se;) {
                        int rs = decode_symbol(bits, ac[c.ta]);
                        if (rs < 0)
                            return false;
                        int r = rs >> 4, sz = rs & 15, value = 0;
                        if (sz) {
                            if (sz != 1)
                                return false;
                            value = bits.bit() ? p1 : m1;
                        } else if (r != 15) {
                            eobrun = (1 << r) + (r ? bits.bits(r) : 0);
                            break;
                        }
                        while (k <= se) {
                            int16_t& v = z[k];
                            if (v != 0) {
                                if (bits.bit() && (v & p1) == 0)
                                    v = int16_t(v >= 0 ? v + p1 : v + m1);
                            } else {
                                if (r == 0) {
                                    if (value)
                                        v = int16_t(value);
                                    k++;
                                    break;
                                }
                                r--;
                            }
                            k++;
                        }
                    }
                }
                if (eobrun > 0) {
                    for (; k <= se; k++) {
                        int16_t& v = z[k];
                        if (v != 0 && bits.bit() && (v & p1) == 0)
                            v = int16_t(v >= 0 ? v + p1 : v + m1);
                    }
                    eobrun--;
                }
                return true;
            };
            int coef[64];
            auto block = [&](Component& c, int bx, int by) {
                std::fill(coef, coef + 64, 0);
                int t = decode_symbol(bits, dc[c.td]);
                if (t < 0 || t > 11)
                    return false;
                c.dc += extend(bits.bits(t), t);
                const uint16_t* q = quant[c.tq];
                coef[0] = c.dc * q[0];
                for (int k = 1; k < 64;) {
                    int rs = decode_symbol(bits, ac[c.ta]);
                    if (rs < 0)
                        return false;
                    int r = rs >> 4, sz = rs & 15;
                    if (sz == 0) {
                        if (r != 15)
                            break;  // end of block
                        k += 16;
                        continue;
                    }
                    k += r;
                    if (k > 63)
                        return false;
                    coef[kZigzag[k]] = extend(bits.bits(sz), sz) * q[kZigzag[k]];
                    k++;
                }
                int stride = c.bw * 8;
                if (bx < c.bw && by < c.bh)
                    idct.run(coef, &c.plane[size_t(by) * 8 * stride + size_t(bx) * 8], stride);
                return true;
            };
            bool interleaved = ns > 1;
            int mcux = (width + 8 * hmax - 1) / (8 * hmax), mcuy = (height + 8 * vmax - 1) / (8 * vmax);
            int units_x, units_y;
            if (interleaved) {
                units_x = mcux;
                units_y = mcuy;
            } else {  // one component: its own blocks, only those covering the image
                Component& c = *sc[0];
                units_x = ((width * c.h + hmax - 1) / hmax + 7) / 8;
                units_y = ((height * c.v + vmax - 1) / vmax + 7) / 8;
            }
            for (auto* c : sc)
                c->dc = 0;
            int todo = restart;
            for (int uy = 0; uy < units_y; uy++)
                for (int ux = 0; ux < units_x; ux++) {
                    if (restart && todo == 0) {
                        // expect RSTn: skip to it and past it
                        size_t p = bits.pos;
                        while (p + 1 < bits.n && !(bits.p[p] == 0xff && bits.p[p + 1] >= 0xd0 && bits.p[p + 1] <= 0xd7))
                            p++;
                        bits.pos = std::min(bits.n, p + 2);
                        bits.reset();
                        for (auto* c : sc)
                            c->dc = 0;
                        eobrun = 0;
                        todo = restart;
                    }
                    auto one = [&](Component& c, int bx, int by) {
                        return progressive ? prog_block(c, bx, by) : block(c, bx, by);
                    };
                    if (interleaved) {
                        for (auto* c : sc)
                            for (int v = 0; v < c->v; v++)
                                for (int h = 0; h < c->h; h++)
                                    if (!one(*c, ux * c->h + h, uy * c->v + v))
                                        return corrupt("entropy-coded data");
                    } else if (!one(*sc[0], ux, uy)) {
                        return corrupt("entropy-coded data");
                    }
                    if (restart)
                        todo--;
                }
            pos += bits.pos;
            continue;
        }
        pos += 2 + len;
    }
    if (!frame)
        return corrupt("no frame");
    if (progressive) {
        int coef[64];
        for (auto& c : comps) {
            const uint16_t* q = quant[c.tq];
            int stride = c.bw * 8;
            for (int by = 0; by < c.bh; by++)
                for (int bx = 0; bx < c.bw; bx++) {
                    const int16_t* z = &c.coef[(size_t(by) * c.bw + size_t(bx)) * 64];
                    for (int k = 0; k < 64; k++)
                        coef[kZigzag[k]] = z[k] * q[kZigzag[k]];
                    idct.run(coef, &c.plane[size_t(by) * 8 * stride + size_t(bx) * 8], stride);
                }
        }
    }
    out.width = width;
    out.height = height;
    out.channels = int(comps.size()) == 1 ? 1 : 3;
    out.rgba.assign(size_t(width) * height * 4, 255);
    std::vector<std::vector<uint8_t>> full(comps.size());
    for (size_t c = 0; c < comps.size(); c++) {
        int sh = hmax / comps[c].h, sv = vmax / comps[c].v;
        upsample(comps[c], sh, sv, width, height, full[c]);
    }
    bool ycc = comps.size() == 3 && !(adobe && adobe_rgb);
    for (size_t k = 0; k < size_t(width) * height; k++) {
        uint8_t* o = &out.rgba[4 * k];
        if (comps.size() == 1) {
            o[0] = o[1] = o[2] = full[0][k];
        } else if (!ycc) {
            o[0] = full[0][k];
            o[1] = full[1][k];
            o[2] = full[2][k];
        } else {
            float y = full[0][k], cb = float(full[1][k]) - 128.0f, cr = float(full[2][k]) - 128.0f;
            auto clamp8 = [](float v) { return uint8_t(std::clamp(int(std::lround(v)), 0, 255)); };
            o[0] = clamp8(y + 1.402f * cr);
            o[1] = clamp8(y - 0.344136f * cb - 0.714136f * cr);
            o[2] = clamp8(y + 1.772f * cb);
        }
    }
    return true;
}

}  // namespace mypbr_host
