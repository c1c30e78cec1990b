// Minimal PNG codec for depth images, written from the PNG specification
// (ISO/IEC 15948) over zlib: chunk parsing with CRC checks, inflate, the five
// scanline filters (None, Sub, Up, Average, Paeth); non-interlaced 8- or
// 16-bit grayscale (Kinect v1 depth in millimetres) and 8-bit RGBA (the
// Kinect v2 tools store each float depth's four bytes as one RGBA pixel).
// The writers use filter None.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace png16 {

// Reads path into pixels (row-major, height x width; 8-bit images widened).
// Returns false with a message in err.
bool read(const std::string& path, std::vector<uint16_t>& pixels, int& width, int& height, std::string& err);
bool write(const std::string& path, const uint16_t* pixels, int width, int height, std::string& err);
// 8-bit RGBA: rgba holds height x width x 4 bytes in the file's R, G, B, A order.
bool read_rgba8(const std::string& path, std::vector<unsigned char>& rgba, int& width, int& height,
                std::string& err);
bool write_rgba8(const std::string& path, const unsigned char* rgba, int width, int height, std::string& err);

}  // namespace png16
