// PNG reading and writing for the host side: the texture decode the
// reference does through Qt (Texture::load, src/scene/texture.cpp:5-31:
// QImage(file).convertToFormat(Format_RGBA8888), then pixelColor) and the
// image file QImage::save writes for a .png output (src/cmd/cmd.cpp:112).
//
// The decoder implements the zlib container (RFC 1950), DEFLATE (RFC 1951:
// stored, fixed and dynamic Huffman blocks) and PNG (ISO/IEC 15948): all
// colour types, bit depths 1-16, the five scanline filters, Adam7
// interlacing, PLTE and tRNS. Output is 8-bit RGBA, row 0 at the top;
// samples of 16-bit images keep their high byte, lower depths are scaled to
// 0..255 as PNG specifies. No gamma correction is applied (Qt applies none
// unless asked to).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace nr {

// Decodes a PNG file held in memory. Returns an empty string on success or
// an error message.
std::string png_decode(const std::vector<uint8_t>& file, int& width, int& height, std::vector<uint8_t>& rgba);

// Decodes a JPEG file held in memory (baseline, extended sequential or
// progressive Huffman, 8-bit, 1 or 3 components) to 8-bit RGB, row 0 at
// the top. Returns an empty string on success or an error message.
std::string jpeg_decode(const std::vector<uint8_t>& file, int& width, int& height, std::vector<uint8_t>& rgb);

// zlib stream -> bytes (exposed for tests), at most `limit` of them.
// Returns "" or an error message.
std::string zlib_inflate(const uint8_t* data, size_t n, std::vector<uint8_t>& out, size_t limit = (size_t)-1);

// 8-bit RGB image (row 0 at the top) -> PNG file bytes (colour type 2,
// filter 0, DEFLATE stored blocks).
std::vector<uint8_t> png_encode_rgb8(const uint8_t* rgb, int width, int height);

// CRC-32 of PNG chunks (ISO 3309 polynomial, reflected).
uint32_t crc32_png(const uint8_t* p, size_t n, uint32_t crc = 0);

}  // namespace nr
