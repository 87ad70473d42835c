// Decoding of 8-bit image files for textures: PNG, TGA, JPEG, BMP, GIF and
// binary PGM / PPM, to RGBA bytes.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace mypbr_host {

// An 8-bit image as RGBA bytes, rows from the top, with the number of
// channels the file holds as stb_image counts them (1 grey, 2 grey + alpha,
// 3 RGB, 4 RGBA; a PNG tRNS chunk adds an alpha channel).
struct LdrImage {
    int width = 0, height = 0, channels = 0;
    std::vector<uint8_t> rgba;
    bool unsupported = false;  // decoding failed on a variant of the format that is not read here

};

bool decode_png(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);
bool decode_tga(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);
bool decode_jpeg(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);
bool decode_bmp(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);
bool decode_pnm(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);
bool decode_gif(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);

// The kind of image file the bytes start with.
enum class ImageKind { Png, Hdr, Jpeg, Bmp, Gif, Pnm, Psd, Pic, Other };
ImageKind sniff_image(const uint8_t* bytes, size_t size);

bool read_file_bytes(const std::string& path, std::vector<uint8_t>& bytes);

// An 8-bit image file (PNG, JPEG, BMP, GIF, PGM / PPM, or TGA as the fallback for files
// no signature names, as stb_image tries it last).
bool read_ldr_image(const std::string& path, LdrImage& out, std::string& error);
bool decode_ldr_image(const uint8_t* bytes, size_t size, LdrImage& out, std::string& error);

}  // namespace mypbr_host
