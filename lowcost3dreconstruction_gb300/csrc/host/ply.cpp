// PLY reader/writer for lcr_point clouds (host code, part of liblcr).
//
// Reads ascii, binary_little_endian and binary_big_endian files with any vertex
// property layout: the fields pcl::io::loadPLYFile maps into PointXYZRGBNormal
// (x y z, nx|normal_x ..., red|r green|g blue|b alpha|a, packed float/uint rgb
// or rgba, curvature) are picked up, everything else -- other vertex
// properties, other elements such as PCL's camera element or face lists -- is
// parsed and skipped.  Writes binary_little_endian with PCL's field order for
// PointXYZRGBNormal (x y z, rgb as red/green/blue, normal_x/y/z, curvature), as
// pcl::io::savePLYFileBinary does for the reference tools.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../../include/lcr.h"

namespace {

enum class T { I8, U8, I16, U16, I32, U32, F32, F64, BAD };

T parse_type(const std::string& s) {
  if (s == "char" || s == "int8") return T::I8;
  if (s == "uchar" || s == "uint8") return T::U8;
  if (s == "short" || s == "int16") return T::I16;
  if (s == "ushort" || s == "uint16") return T::U16;
  if (s == "int" || s == "int32") return T::I32;
  if (s == "uint" || s == "uint32") return T::U32;
  if (s == "float" || s == "float32") return T::F32;
  if (s == "double" || s == "float64") return T::F64;
  return T::BAD;
}

size_t type_size(T t) {
  switch (t) {
    case T::I8: case T::U8: return 1;
    case T::I16: case T::U16: return 2;
    case T::I32: case T::U32: case T::F32: return 4;
    case T::F64: return 8;
    default: return 0;
  }
}

enum Field { F_NONE, F_X, F_Y, F_Z, F_NX, F_NY, F_NZ, F_R, F_G, F_B, F_A, F_RGB, F_RGBA, F_CURV };

Field vertex_field(const std::string& n) {
  if (n == "x") return F_X;
  if (n == "y") return F_Y;
  if (n == "z") return F_Z;
  if (n == "nx" || n == "normal_x") return F_NX;
  if (n == "ny" || n == "normal_y") return F_NY;
  if (n == "nz" || n == "normal_z") return F_NZ;
  if (n == "red" || n == "r" || n == "diffuse_red") return F_R;
  if (n == "green" || n == "g" || n == "diffuse_green") return F_G;
  if (n == "blue" || n == "b" || n == "diffuse_blue") return F_B;
  if (n == "alpha" || n == "a") return F_A;
  if (n == "rgb") return F_RGB;
  if (n == "rgba") return F_RGBA;
  if (n == "curvature") return F_CURV;
  return F_NONE;
}

struct Prop {
  std::string name;
  T type = T::BAD;
  bool list = false;
  T count_type = T::BAD;
  Field field = F_NONE;
};

struct Element {
  std::string name;
  size_t count = 0;
  std::vector<Prop> props;
};

inline void swap_bytes(unsigned char* p, size_t n) {
  for (size_t i = 0; i < n / 2; ++i) std::swap(p[i], p[n - 1 - i]);
}

// Value of a binary scalar, as double, plus its raw 32-bit pattern (for packed rgb).
bool read_bin(std::istream& in, T t, bool big, double& v, uint32_t& raw) {
  unsigned char b[8];
  const size_t n = type_size(t);
  if (!in.read(reinterpret_cast<char*>(b), static_cast<std::streamsize>(n))) return false;
  if (big) swap_bytes(b, n);
  raw = 0;
  switch (t) {
    case T::I8: { int8_t x; std::memcpy(&x, b, 1); v = x; raw = static_cast<uint8_t>(x); break; }
    case T::U8: { uint8_t x; std::memcpy(&x, b, 1); v = x; raw = x; break; }
    case T::I16: { int16_t x; std::memcpy(&x, b, 2); v = x; raw = static_cast<uint16_t>(x); break; }
    case T::U16: { uint16_t x; std::memcpy(&x, b, 2); v = x; raw = x; break; }
    case T::I32: { int32_t x; std::memcpy(&x, b, 4); v = x; std::memcpy(&raw, b, 4); break; }
    case T::U32: { uint32_t x; std::memcpy(&x, b, 4); v = x; raw = x; break; }
    case T::F32: { float x; std::memcpy(&x, b, 4); v = x; std::memcpy(&raw, b, 4); break; }
    case T::F64: { double x; std::memcpy(&x, b, 8); v = x; float f = static_cast<float>(x); std::memcpy(&raw, &f, 4); break; }
    default: return false;
  }
  return true;
}

bool read_ascii(std::istream& in, T t, double& v, uint32_t& raw) {
  std::string tok;
  if (!(in >> tok)) return false;
  errno = 0;
  char* end = nullptr;
  if (t == T::F32) {
    const float f = std::strtof(tok.c_str(), &end);  // one rounding, as PCL's text parse to float
    v = f;
    std::memcpy(&raw, &f, 4);
  } else if (t == T::F64) {
    v = std::strtod(tok.c_str(), &end);
    const float f = static_cast<float>(v);
    std::memcpy(&raw, &f, 4);
  } else {
    const long long x = std::strtoll(tok.c_str(), &end, 10);
    v = static_cast<double>(x);
    raw = static_cast<uint32_t>(x);
  }
  return end && *end == '\0';
}

void assign(lcr_point& p, Field f, T t, double v, uint32_t raw) {
  switch (f) {
    case F_X: p.x = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_Y: p.y = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_Z: p.z = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_NX: p.normal_x = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_NY: p.normal_y = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_NZ: p.normal_z = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_CURV: p.curvature = t == T::F32 ? *reinterpret_cast<float*>(&raw) : static_cast<float>(v); break;
    case F_R: p.r = static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v)); break;
    case F_G: p.g = static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v)); break;
    case F_B: p.b = static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v)); break;
    case F_A: p.a = static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v)); break;
    case F_RGB:
    case F_RGBA:  // packed 0xAARRGGBB (float bit pattern or integer)
      p.b = static_cast<uint8_t>(raw & 255u);
      p.g = static_cast<uint8_t>((raw >> 8) & 255u);
      p.r = static_cast<uint8_t>((raw >> 16) & 255u);
      p.a = static_cast<uint8_t>((raw >> 24) & 255u);
      break;
    default: break;
  }
}

thread_local std::string g_ply_error;

lcr_status fail(lcr_status s, const std::string& msg) {
  g_ply_error = msg;
  return s;
}

}  // namespace

extern "C" {

LCR_API const char* lcr_ply_last_error(void) { return g_ply_error.c_str(); }

LCR_API void lcr_free(void* p) { std::free(p); }

LCR_API lcr_status lcr_ply_read(const char* path, lcr_point** out, size_t* n_out) {
  if (!path || !out || !n_out) return fail(LCR_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  *n_out = 0;
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(LCR_ERR_IO, std::string("cannot open ") + path);
  std::string line;
  if (!std::getline(in, line) || line.rfind("ply", 0) != 0) return fail(LCR_ERR_IO, "not a PLY file");
  int format = -1;  // 0 ascii, 1 binary le, 2 binary be
  std::vector<Element> els;
  while (std::getline(in, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ls(line);
    std::string kw;
    ls >> kw;
    if (kw == "format") {
      std::string f;
      ls >> f;
      format = f == "ascii" ? 0 : f == "binary_little_endian" ? 1 : f == "binary_big_endian" ? 2 : -1;
      if (format < 0) return fail(LCR_ERR_IO, "unknown PLY format " + f);
    } else if (kw == "element") {
      Element e;
      ls >> e.name >> e.count;
      els.push_back(e);
    } else if (kw == "property") {
      if (els.empty()) return fail(LCR_ERR_IO, "property before element");
      Prop p;
      std::string t;
      ls >> t;
      if (t == "list") {
        std::string ct, it;
        ls >> ct >> it >> p.name;
        p.list = true;
        p.count_type = parse_type(ct);
        p.type = parse_type(it);
        if (p.count_type == T::BAD || p.type == T::BAD) return fail(LCR_ERR_IO, "bad list property");
      } else {
        ls >> p.name;
        p.type = parse_type(t);
        if (p.type == T::BAD) return fail(LCR_ERR_IO, "bad property type " + t);
      }
      if (els.back().name == "vertex" && !p.list) p.field = vertex_field(p.name);
      els.back().props.push_back(p);
    } else if (kw == "end_header") {
      break;
    }
  }
  if (format < 0) return fail(LCR_ERR_IO, "missing format line");
  size_t nv = 0;
  for (const Element& e : els)
    if (e.name == "vertex") nv = e.count;
  if (nv > (static_cast<size_t>(1) << 31)) return fail(LCR_ERR_IO, "vertex count too large");
  lcr_point* pts = static_cast<lcr_point*>(std::calloc(nv ? nv : 1, sizeof(lcr_point)));
  if (!pts) return fail(LCR_ERR_OOM, "allocation failed");
  const bool big = format == 2;
  for (const Element& e : els) {
    const bool isv = e.name == "vertex";
    for (size_t i = 0; i < e.count; ++i) {
      lcr_point dummy;
      lcr_point& p = isv ? pts[i] : dummy;
      for (const Prop& pr : e.props) {
        double v;
        uint32_t raw;
        if (pr.list) {
          bool ok = format == 0 ? read_ascii(in, pr.count_type, v, raw) : read_bin(in, pr.count_type, big, v, raw);
          if (!ok || v < 0) { std::free(pts); return fail(LCR_ERR_IO, "truncated list"); }
          const size_t cnt = static_cast<size_t>(v);
          for (size_t k = 0; k < cnt; ++k) {
            ok = format == 0 ? read_ascii(in, pr.type, v, raw) : read_bin(in, pr.type, big, v, raw);
            if (!ok) { std::free(pts); return fail(LCR_ERR_IO, "truncated list data"); }
          }
          continue;
        }
        const bool ok = format == 0 ? read_ascii(in, pr.type, v, raw) : read_bin(in, pr.type, big, v, raw);
        if (!ok) {
          std::free(pts);
          return fail(LCR_ERR_IO, "truncated or malformed " + e.name + " data");
        }
        if (isv) assign(p, pr.field, pr.type, v, raw);
      }
    }
  }
  *out = pts;
  *n_out = nv;
  return LCR_OK;
}

LCR_API lcr_status lcr_ply_write(const char* path, const lcr_point* pts, size_t n, int binary) {
  if (!path || (!pts && n)) return fail(LCR_ERR_INVALID_ARG, "null argument");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(LCR_ERR_IO, std::string("cannot create ") + path);
  std::fprintf(f, "ply\nformat %s 1.0\ncomment lcr generated\nelement vertex %zu\n",
               binary ? "binary_little_endian" : "ascii", n);
  std::fprintf(f,
               "property float x\nproperty float y\nproperty float z\nproperty uchar red\nproperty uchar green\n"
               "property uchar blue\nproperty float normal_x\nproperty float normal_y\nproperty float normal_z\n"
               "property float curvature\nend_header\n");
  bool ok = true;
  if (binary) {
    std::vector<unsigned char> buf(n * 31);
    for (size_t i = 0; i < n; ++i) {
      unsigned char* b = &buf[i * 31];
      const lcr_point& p = pts[i];
      std::memcpy(b, &p.x, 4);
      std::memcpy(b + 4, &p.y, 4);
      std::memcpy(b + 8, &p.z, 4);
      b[12] = p.r;
      b[13] = p.g;
      b[14] = p.b;
      std::memcpy(b + 15, &p.normal_x, 4);
      std::memcpy(b + 19, &p.normal_y, 4);
      std::memcpy(b + 23, &p.normal_z, 4);
      std::memcpy(b + 27, &p.curvature, 4);
    }
    ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  } else {
    for (size_t i = 0; i < n && ok; ++i) {
      const lcr_point& p = pts[i];
      ok = std::fprintf(f, "%.9g %.9g %.9g %d %d %d %.9g %.9g %.9g %.9g\n", p.x, p.y, p.z, p.r, p.g, p.b, p.normal_x,
                        p.normal_y, p.normal_z, p.curvature) > 0;
    }
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? LCR_OK : fail(LCR_ERR_IO, std::string("write failed: ") + path);
}

}  // extern "C"
