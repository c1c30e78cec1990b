// Minimal PNG codec for depth images: 8- or 16-bit grayscale, non-interlaced,
// written from the PNG specification (ISO/IEC 15948) over zlib: chunk
// parsing with CRC checks, inflate, the five scanline filters (None, Sub, Up,
// Average, Paeth); the writer emits 16-bit grayscale with filter None.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace png16 {

// Reads path into pixels (row-major, height x width; 8-bit images widened).
// Returns false with a message in err.
bool read(const std::string& path, std::vector<uint16_t>& pixels, int& width, int& height, std::string& err);
bool write(const std::string& path, const uint16_t* pixels, int width, int height, std::string& err);

}  // namespace png16
