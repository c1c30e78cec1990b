// PNG codec for depth images (see png16.h).
#include "png16.h"

#include <zlib.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace png16 {
namespace {

const unsigned char kSig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};

uint32_t be32(const unsigned char* p) {
  return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) | (static_cast<uint32_t>(p[2]) << 8) | p[3];
}

void put32(std::vector<unsigned char>& o, uint32_t v) {
  o.push_back(static_cast<unsigned char>(v >> 24));
  o.push_back(static_cast<unsigned char>(v >> 16));
  o.push_back(static_cast<unsigned char>(v >> 8));
  o.push_back(static_cast<unsigned char>(v));
}

void chunk(std::vector<unsigned char>& o, const char* type, const unsigned char* data, size_t n) {
  put32(o, static_cast<uint32_t>(n));
  const size_t at = o.size();
  o.insert(o.end(), type, type + 4);
  o.insert(o.end(), data, data + n);
  put32(o, static_cast<uint32_t>(crc32(0L, o.data() + at, static_cast<uInt>(n + 4))));
}

int paeth(int a, int b, int c) {
  const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

}  // namespace

namespace {

// The unfiltered image bytes of path (height rows of width * channels *
// depth / 8 bytes) and its header; false with a message in err.
bool decode(const std::string& path, std::vector<unsigned char>& img, int& width, int& height, int& depth,
            int& ctype, std::string& err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open " + path;
    return false;
  }
  std::vector<unsigned char> buf;
  unsigned char tmp[65536];
  size_t got;
  while ((got = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  std::fclose(f);
  if (buf.size() < 8 || std::memcmp(buf.data(), kSig, 8) != 0) {
    err = path + " is not a PNG file";
    return false;
  }
  size_t p = 8;
  int interlace = 0;
  depth = 0;
  ctype = -1;
  std::vector<unsigned char> idat;
  bool have_hdr = false, ended = false;
  while (p + 12 <= buf.size() && !ended) {
    const uint32_t n = be32(&buf[p]);
    if (p + 12 + static_cast<size_t>(n) > buf.size()) break;
    const unsigned char* type = &buf[p + 4];
    const unsigned char* data = &buf[p + 8];
    if (static_cast<uint32_t>(crc32(0L, type, n + 4)) != be32(data + n)) {
      err = path + ": chunk CRC mismatch";
      return false;
    }
    if (!std::memcmp(type, "IHDR", 4) && n >= 13) {
      width = static_cast<int>(be32(data));
      height = static_cast<int>(be32(data + 4));
      depth = data[8];
      ctype = data[9];
      interlace = data[12];
      have_hdr = true;
    } else if (!std::memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), data, data + n);
    } else if (!std::memcmp(type, "IEND", 4)) {
      ended = true;
    }
    p += 12 + n;
  }
  if (!have_hdr || !ended) {
    err = path + ": truncated PNG";
    return false;
  }
  const int channels = ctype == 0 ? 1 : ctype == 6 ? 4 : 0;
  if (channels == 0 || (depth != 8 && depth != 16) || interlace != 0 || width <= 0 || height <= 0 ||
      static_cast<long long>(width) * height > (1LL << 28)) {
    err = path + ": only non-interlaced 8- or 16-bit grayscale or RGBA PNG is supported";
    return false;
  }
  const size_t bpp = static_cast<size_t>(channels) * depth / 8, stride = static_cast<size_t>(width) * bpp;
  std::vector<unsigned char> raw((stride + 1) * height);
  uLongf rawlen = static_cast<uLongf>(raw.size());
  if (uncompress(raw.data(), &rawlen, idat.data(), static_cast<uLong>(idat.size())) != Z_OK || rawlen != raw.size()) {
    err = path + ": corrupt image data";
    return false;
  }
  img.assign(stride * height, 0);
  const std::vector<unsigned char> zero(stride, 0);
  for (int y = 0; y < height; ++y) {
    const unsigned char* x = &raw[y * (stride + 1) + 1];
    const unsigned char* b = y > 0 ? &img[(y - 1) * stride] : zero.data();  // the row above
    unsigned char* cur = &img[y * stride];
    // one loop per filter type; a = the byte bpp to the left, c = the one above it
    switch (raw[y * (stride + 1)]) {
      case 0:
        std::memcpy(cur, x, stride);
        break;
      case 1:
        for (size_t i = 0; i < stride; ++i) cur[i] = static_cast<unsigned char>(x[i] + (i >= bpp ? cur[i - bpp] : 0));
        break;
      case 2:
        for (size_t i = 0; i < stride; ++i) cur[i] = static_cast<unsigned char>(x[i] + b[i]);
        break;
      case 3:
        for (size_t i = 0; i < stride; ++i)
          cur[i] = static_cast<unsigned char>(x[i] + (((i >= bpp ? cur[i - bpp] : 0) + b[i]) >> 1));
        break;
      case 4:
        for (size_t i = 0; i < stride; ++i)
          cur[i] = static_cast<unsigned char>(
              x[i] + (i >= bpp ? paeth(cur[i - bpp], b[i], b[i - bpp]) : paeth(0, b[i], 0)));
        break;
      default:
        err = path + ": unknown scanline filter";
        return false;
    }
  }
  return true;
}

// Writes rows of stride bytes with filter None under the given header.
bool encode(const std::string& path, const unsigned char* img, size_t stride, int width, int height, int depth,
            int ctype, std::string& err) {
  std::vector<unsigned char> raw((stride + 1) * height);
  for (int y = 0; y < height; ++y) {
    raw[y * (stride + 1)] = 0;
    std::memcpy(&raw[y * (stride + 1) + 1], img + y * stride, stride);
  }
  uLongf zlen = compressBound(static_cast<uLong>(raw.size()));
  std::vector<unsigned char> z(zlen);
  if (compress2(z.data(), &zlen, raw.data(), static_cast<uLong>(raw.size()), 6) != Z_OK) {
    err = "compression failed";
    return false;
  }
  std::vector<unsigned char> out(kSig, kSig + 8);
  const uint32_t w = static_cast<uint32_t>(width), h = static_cast<uint32_t>(height);
  const unsigned char hdr[13] = {static_cast<unsigned char>(w >> 24), static_cast<unsigned char>(w >> 16),
                                 static_cast<unsigned char>(w >> 8),  static_cast<unsigned char>(w),
                                 static_cast<unsigned char>(h >> 24), static_cast<unsigned char>(h >> 16),
                                 static_cast<unsigned char>(h >> 8),  static_cast<unsigned char>(h),
                                 static_cast<unsigned char>(depth), static_cast<unsigned char>(ctype), 0, 0, 0};
  chunk(out, "IHDR", hdr, 13);
  chunk(out, "IDAT", z.data(), zlen);
  chunk(out, "IEND", nullptr, 0);
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    err = "cannot create " + path;
    return false;
  }
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  return (std::fclose(f) == 0) && ok ? true : (err = "write failed: " + path, false);
}

}  // namespace

bool read(const std::string& path, std::vector<uint16_t>& pixels, int& width, int& height, std::string& err) {
  std::vector<unsigned char> img;
  int depth = 0, ctype = 0;
  if (!decode(path, img, width, height, depth, ctype, err)) return false;
  if (ctype != 0) {
    err = path + ": not a grayscale PNG";
    return false;
  }
  const size_t n = static_cast<size_t>(width) * height;
  pixels.resize(n);
  for (size_t i = 0; i < n; ++i)
    pixels[i] = depth == 16 ? static_cast<uint16_t>((img[2 * i] << 8) | img[2 * i + 1]) : img[i];
  return true;
}

bool read_rgba8(const std::string& path, std::vector<unsigned char>& rgba, int& width, int& height,
                std::string& err) {
  int depth = 0, ctype = 0;
  if (!decode(path, rgba, width, height, depth, ctype, err)) return false;
  if (ctype != 6 || depth != 8) {
    err = path + ": not an 8-bit RGBA PNG";
    return false;
  }
  return true;
}

bool write_rgba8(const std::string& path, const unsigned char* rgba, int width, int height, std::string& err) {
  return encode(path, rgba, static_cast<size_t>(width) * 4, width, height, 8, 6, err);
}

bool write(const std::string& path, const uint16_t* pixels, int width, int height, std::string& err) {
  const size_t n = static_cast<size_t>(width) * height;
  std::vector<unsigned char> img(2 * n);
  for (size_t i = 0; i < n; ++i) {
    img[2 * i] = static_cast<unsigned char>(pixels[i] >> 8);
    img[2 * i + 1] = static_cast<unsigned char>(pixels[i] & 255);
  }
  return encode(path, img.data(), static_cast<size_t>(width) * 2, width, height, 16, 0, err);
}

}  // namespace png16
