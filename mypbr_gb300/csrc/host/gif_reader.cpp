// GIF decoding (the first frame, to RGBA bytes) as stb_image v2.30 decodes
// it for `image_texture` (texture.h:78 calls stbi_load with 4 channels):
//
//  * the channel count is always 4;
//  * the canvas starts transparent black; the first image descriptor's
//    rectangle is drawn into it with the local color table, else the global
//    one; an index whose entry is transparent (the graphic control
//    extension's transparent index) or lies past the table's entries leaves
//    the canvas as it is;
//  * when the background index is above 0, canvas pixels the image did not
//    cover take the global table's background color, opaque, with red and
//    blue exchanged (stb copies the entry in its blue-first storage order);
//  * LZW codes follow the GIF 89a specification (a clear code must come
//    first; code width grows when the next free code reaches a power of two,
//    up to 12 bits, and the table keeps growing past 4096 entries without a
//    clear code, as stb's does, up to 8192), pixels past the rectangle are
//    dropped, and interlaced images fill rows in the four-pass order;
//  * bytes past the end of the file read as 0, so a file cut inside its
//    image data decodes to the part before the cut (as stb's reader does).

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "image_reader.h"

namespace mypbr_host {

namespace {

struct ByteReader {
    const uint8_t* b;
    size_t n, pos = 0;
    int get() { return pos < n ? b[pos++] : 0; }
    int get16() {
        int lo = get();
        return lo | get() << 8;
    }
    void skip(size_t k) { pos = k > n - std::min(pos, n) ? n : pos + k; }
};

}  // namespace

bool decode_gif(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error) {
    error = "not a readable GIF image";
    if (size < 6 || std::memcmp(bytes, "GIF8", 4) != 0 || (bytes[4] != '7' && bytes[4] != '9') || bytes[5] != 'a')
        return false;
    ByteReader r{bytes, size, 6};
    const int W = r.get16(), H = r.get16();
    const int flags = r.get(), bg_index = r.get();
    r.get();  // aspect ratio
    if (W <= 0 || H <= 0 || W > (1 << 15) || H > (1 << 15)) {
        error = "GIF image of " + std::to_string(W) + "x" + std::to_string(H) + " is not supported";
        return false;
    }
    uint8_t global[256][4] = {}, local[256][4] = {};
    auto read_table = [&](uint8_t table[256][4], int entries, int transparent) {
        for (int i = 0; i < entries; i++) {
            table[i][0] = uint8_t(r.get());
            table[i][1] = uint8_t(r.get());
            table[i][2] = uint8_t(r.get());
            table[i][3] = i == transparent ? 0 : 255;
        }
    };
    if (flags & 0x80)
        read_table(global, 2 << (flags & 7), -1);
    int transparent = -1, ext_flags = 0;
    std::vector<uint8_t> px(size_t(W) * size_t(H) * 4, 0);
    for (;;) {
        const int tag = r.get();
        if (tag == 0x21) {  // extension
            const int kind = r.get();
            if (kind == 0xF9) {  // graphic control
                const int len = r.get();
                if (len != 4) {
                    error = "GIF graphic control extension of " + std::to_string(len) + " bytes";
                    return false;
                }
                ext_flags = r.get();
                r.get16();  // delay
                if (transparent >= 0)
                    global[transparent][3] = 255;
                if (ext_flags & 1) {
                    transparent = r.get();
                    global[transparent][3] = 0;
                } else {
                    r.get();
                    transparent = -1;
                }
            }
            for (int len = r.get(); len != 0; len = r.get())
                r.skip(size_t(len));
            continue;
        }
        if (tag == 0x3B) {
            error = "GIF file holds no image";
            return false;
        }
        if (tag != 0x2C) {
            error = "GIF block of unknown kind " + std::to_string(tag);
            return false;
        }
        // image descriptor: the first image is the texture
        const int x0 = r.get16(), y0 = r.get16(), w = r.get16(), h = r.get16();
        if (x0 + w > W || y0 + h > H) {
            error = "GIF image rectangle outside the canvas";
            return false;
        }
        const int lflags = r.get();
        const uint8_t(*table)[4] = global;
        if (lflags & 0x80) {
            read_table(local, 2 << (lflags & 7), (ext_flags & 1) ? transparent : -1);
            table = local;
        } else if (!(flags & 0x80)) {
            error = "GIF image without a color table";
            return false;
        }
        std::vector<uint8_t> drawn(size_t(W) * size_t(H), 0);
        // rows in drawing order: plain, or interlaced passes (every 8th from
        // 0, every 8th from 4, every 4th from 2, every 2nd from 1)
        std::vector<int> rows;
        if (lflags & 0x40) {
            static const int start[4] = {0, 4, 2, 1}, step[4] = {8, 8, 4, 2};
            for (int p = 0; p < 4; p++)
                for (int y = start[p]; y < h; y += step[p])
                    rows.push_back(y);
        } else {
            for (int y = 0; y < h; y++)
                rows.push_back(y);
        }
        size_t emitted = 0;
        const size_t total = w > 0 ? size_t(w) * size_t(h) : 0;
        auto emit = [&](int index) {
            if (emitted >= total)
                return;
            const int y = y0 + rows[emitted / size_t(w)], x = x0 + int(emitted % size_t(w));
            emitted++;
            const size_t k = size_t(y) * size_t(W) + size_t(x);
            drawn[k] = 1;
            const uint8_t* c = table[index];
            if (c[3] > 128)
                std::memcpy(&px[4 * k], c, 4);
        };
        // LZW
        const int min_size = r.get();
        if (min_size > 12) {
            error = "GIF code size above 12 bits";
            return false;
        }
        const int clear = 1 << min_size;
        struct Code {
            int16_t prefix;
            uint8_t first, suffix;
        };
        std::vector<Code> codes(8192);
        for (int c = 0; c < clear; c++)
            codes[c] = Code{-1, uint8_t(c), uint8_t(c)};
        int size_bits = min_size + 1, mask = (1 << size_bits) - 1, avail = clear + 2, old = -1;
        bool seen_clear = false;
        uint32_t bits = 0;
        int have = 0, block = 0;
        std::vector<uint8_t> chain;
        for (;;) {
            if (have < size_bits) {
                if (block == 0) {
                    block = r.get();
                    if (block == 0)
                        break;  // end of the image data
                }
                block--;
                bits |= uint32_t(r.get()) << have;
                have += 8;
                continue;
            }
            const int code = int(bits & uint32_t(mask));
            bits >>= size_bits;
            have -= size_bits;
            if (code == clear) {
                size_bits = min_size + 1;
                mask = (1 << size_bits) - 1;
                avail = clear + 2;
                old = -1;
                seen_clear = true;
                continue;
            }
            if (code == clear + 1)
                break;  // end of information
            if (code > avail) {
                error = "GIF image data holds an undefined code";
                return false;
            }
            if (!seen_clear) {
                error = "GIF image data does not start with a clear code";
                return false;
            }
            if (old >= 0) {
                if (avail >= 8192) {
                    error = "GIF image data overflows the code table";
                    return false;
                }
                Code& e = codes[avail++];
                e.prefix = int16_t(old);
                e.first = codes[old].first;
                e.suffix = codes[code].first;  // the new entry itself when code == avail
            } else if (code == avail) {
                error = "GIF image data holds an undefined code";
                return false;
            }
            chain.clear();
            for (int c = code; c >= 0; c = codes[c].prefix)
                chain.push_back(codes[c].suffix);
            for (size_t i = chain.size(); i-- > 0;)
                emit(chain[i]);
            if ((avail & mask) == 0 && avail <= 0x0FFF) {
                size_bits++;
                mask = (1 << size_bits) - 1;
            }
            old = code;
        }
        if (bg_index > 0) {
            // stb copies its table entry, stored blue first, as it stands: the
            // background's red and blue come out exchanged
            uint8_t bg[4] = {global[bg_index][2], global[bg_index][1], global[bg_index][0], 255};
            for (size_t k = 0; k < drawn.size(); k++)
                if (!drawn[k])
                    std::memcpy(&px[4 * k], bg, 4);
        }
        out.width = W;
        out.height = H;
        out.channels = 4;
        out.rgba = std::move(px);
        error.clear();
        return true;
    }
}

}  // namespace mypbr_host
