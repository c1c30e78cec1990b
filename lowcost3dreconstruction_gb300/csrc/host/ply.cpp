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
//
// The file is read in one piece; vertex records decode through the property
// list straight from the buffer, text scalars with std::from_chars (correctly
// rounded, as strtof/strtod), and large clouds split over host threads: text
// files one instance per line in parallel (any other layout falls back to the
// token stream).  The text writer prints the shortest form that reads back to
// the same float (std::to_chars).
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <thread>
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
inline void decode_bin(const unsigned char* src, T t, bool big, double& v, uint32_t& raw) {
  unsigned char b[8];
  const size_t n = type_size(t);
  std::memcpy(b, src, n);
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
    default: v = 0; break;
  }
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Next whitespace-separated token of [p, end).
inline bool next_token(const char*& p, const char* end, const char*& ts, const char*& te) {
  while (p < end && is_space(*p)) ++p;
  if (p >= end) return false;
  ts = p;
  while (p < end && !is_space(*p)) ++p;
  te = p;
  return true;
}

// One text scalar, correctly rounded as strtof/strtod would (from_chars).
inline bool parse_token(const char* s, const char* e, T t, double& v, uint32_t& raw) {
  if (s < e && *s == '+') ++s;
  if (t == T::F32) {
    float f = 0.f;
    const auto r = std::from_chars(s, e, f);
    if (r.ec != std::errc() || r.ptr != e) return false;
    v = f;
    std::memcpy(&raw, &f, 4);
  } else if (t == T::F64) {
    double d = 0.0;
    const auto r = std::from_chars(s, e, d);
    if (r.ec != std::errc() || r.ptr != e) return false;
    v = d;
    const float f = static_cast<float>(d);
    std::memcpy(&raw, &f, 4);
  } else {
    long long x = 0;
    const auto r = std::from_chars(s, e, x);
    if (r.ec != std::errc() || r.ptr != e) return false;
    v = static_cast<double>(x);
    raw = static_cast<uint32_t>(x);
  }
  return true;
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

// Work split over host threads for large element counts (each part a
// contiguous range; f(begin, end, part) returns false on malformed data).
template <class F>
bool parallel_ranges(size_t n, F&& f) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t parts = n >= 65536 ? hw : 1;
  if (parts == 1) return f(size_t{0}, n, size_t{0});
  std::vector<std::thread> th;
  std::vector<char> ok(parts, 1);
  for (size_t k = 0; k < parts; ++k)
    th.emplace_back([&, k] { ok[k] = f(n * k / parts, n * (k + 1) / parts, k) ? 1 : 0; });
  for (auto& t : th) t.join();
  for (char c : ok)
    if (!c) return false;
  return true;
}

bool read_file(const char* path, std::vector<char>& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  bool ok = std::fseek(f, 0, SEEK_END) == 0;
  const long sz = ok ? std::ftell(f) : -1;
  ok = ok && sz >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
  if (ok) {
    buf.resize(static_cast<size_t>(sz));
    ok = sz == 0 || std::fread(buf.data(), 1, buf.size(), f) == buf.size();
  }
  std::fclose(f);
  return ok;
}

}  // namespace

extern "C" {

LCR_API const char* lcr_ply_last_error(void) { return g_ply_error.c_str(); }

LCR_API void lcr_free(void* p) { std::free(p); }

LCR_API lcr_status lcr_ply_read(const char* path, lcr_point** out, size_t* n_out) {
  if (!path || !out || !n_out) return fail(LCR_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  *n_out = 0;
  std::vector<char> file;
  if (!read_file(path, file)) return fail(LCR_ERR_IO, std::string("cannot open ") + path);
  const char* p = file.data();
  const char* const end = p + file.size();
  // ---- header, line by line
  auto next_line = [&](std::string& line) {
    if (p >= end) return false;
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(end - p)));
    const char* le = nl ? nl : end;
    line.assign(p, le);
    if (!line.empty() && line.back() == '\r') line.pop_back();
    p = nl ? nl + 1 : end;
    return true;
  };
  std::string line;
  if (!next_line(line) || line.rfind("ply", 0) != 0) return fail(LCR_ERR_IO, "not a PLY file");
  int format = -1;  // 0 ascii, 1 binary le, 2 binary be
  std::vector<Element> els;
  bool ended = false;
  while (next_line(line)) {
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
      Prop pr;
      std::string t;
      ls >> t;
      if (t == "list") {
        std::string ct, it;
        ls >> ct >> it >> pr.name;
        pr.list = true;
        pr.count_type = parse_type(ct);
        pr.type = parse_type(it);
        if (pr.count_type == T::BAD || pr.type == T::BAD) return fail(LCR_ERR_IO, "bad list property");
      } else {
        ls >> pr.name;
        pr.type = parse_type(t);
        if (pr.type == T::BAD) return fail(LCR_ERR_IO, "bad property type " + t);
      }
      if (els.back().name == "vertex" && !pr.list) pr.field = vertex_field(pr.name);
      els.back().props.push_back(pr);
    } else if (kw == "end_header") {
      ended = true;
      break;
    }
  }
  if (format < 0) return fail(LCR_ERR_IO, "missing format line");
  if (!ended) return fail(LCR_ERR_IO, "missing end_header");
  size_t nv = 0;
  for (const Element& e : els)
    if (e.name == "vertex") nv = e.count;
  if (nv > (static_cast<size_t>(1) << 31)) return fail(LCR_ERR_IO, "vertex count too large");
  lcr_point* pts = static_cast<lcr_point*>(std::calloc(nv ? nv : 1, sizeof(lcr_point)));
  if (!pts) return fail(LCR_ERR_OOM, "allocation failed");
  const bool big = format == 2;
  auto bad = [&](const std::string& msg) {
    std::free(pts);
    return fail(LCR_ERR_IO, msg);
  };
  for (const Element& e : els) {
    const bool isv = e.name == "vertex";
    bool has_list = false;
    for (const Prop& pr : e.props) has_list |= pr.list;
    if (format != 0) {
      // ------------------------------------------------------------ binary
      if (!has_list) {
        size_t rec = 0;
        for (const Prop& pr : e.props) rec += type_size(pr.type);
        if (static_cast<size_t>(end - p) / (rec ? rec : 1) < e.count)
          return bad("truncated or malformed " + e.name + " data");
        if (isv) {
          const unsigned char* base = reinterpret_cast<const unsigned char*>(p);
          parallel_ranges(e.count, [&](size_t b, size_t en, size_t) {
            for (size_t i = b; i < en; ++i) {
              const unsigned char* r = base + i * rec;
              size_t off = 0;
              for (const Prop& pr : e.props) {
                double v;
                uint32_t raw;
                decode_bin(r + off, pr.type, big, v, raw);
                assign(pts[i], pr.field, pr.type, v, raw);
                off += type_size(pr.type);
              }
            }
            return true;
          });
        }
        p += rec * e.count;
      } else {
        for (size_t i = 0; i < e.count; ++i) {
          lcr_point dummy;
          lcr_point& pt = isv ? pts[i] : dummy;
          for (const Prop& pr : e.props) {
            double v;
            uint32_t raw;
            if (pr.list) {
              const size_t cs = type_size(pr.count_type);
              if (static_cast<size_t>(end - p) < cs) return bad("truncated list");
              decode_bin(reinterpret_cast<const unsigned char*>(p), pr.count_type, big, v, raw);
              p += cs;
              if (v < 0) return bad("truncated list");
              const size_t bytes = static_cast<size_t>(v) * type_size(pr.type);
              if (static_cast<size_t>(end - p) < bytes) return bad("truncated list data");
              p += bytes;
              continue;
            }
            const size_t sz = type_size(pr.type);
            if (static_cast<size_t>(end - p) < sz) return bad("truncated or malformed " + e.name + " data");
            decode_bin(reinterpret_cast<const unsigned char*>(p), pr.type, big, v, raw);
            p += sz;
            if (isv) assign(pt, pr.field, pr.type, v, raw);
          }
        }
      }
      continue;
    }
    // -------------------------------------------------------------- ascii
    // Fast form: one instance per line (what every writer produces), lines
    // parsed in parallel; any other layout takes the token stream below.
    bool done = false;
    if (isv && !has_list && e.count > 0) {
      std::vector<const char*> starts(e.count + 1);
      const char* q = p;
      size_t i = 0;
      for (; i < e.count && q < end; ++i) {
        starts[i] = q;
        const char* nl = static_cast<const char*>(std::memchr(q, '\n', static_cast<size_t>(end - q)));
        q = nl ? nl + 1 : end;
      }
      if (i == e.count) {
        starts[e.count] = q;
        const bool ok = parallel_ranges(e.count, [&](size_t b, size_t en, size_t) {
          for (size_t k = b; k < en; ++k) {
            const char* s = starts[k];
            const char* le = starts[k + 1];
            for (const Prop& pr : e.props) {
              const char *ts, *te;
              double v;
              uint32_t raw;
              if (!next_token(s, le, ts, te) || !parse_token(ts, te, pr.type, v, raw)) return false;
              assign(pts[k], pr.field, pr.type, v, raw);
            }
            const char *ts, *te;
            if (next_token(s, le, ts, te)) return false;  // extra tokens: not one instance per line
          }
          return true;
        });
        if (ok) {
          p = q;
          done = true;
        } else {
          std::memset(pts, 0, sizeof(lcr_point) * nv);
        }
      }
    }
    if (done) continue;
    for (size_t i = 0; i < e.count; ++i) {
      lcr_point dummy;
      lcr_point& pt = isv ? pts[i] : dummy;
      for (const Prop& pr : e.props) {
        const char *ts, *te;
        double v;
        uint32_t raw;
        if (pr.list) {
          if (!next_token(p, end, ts, te) || !parse_token(ts, te, pr.count_type, v, raw) || v < 0)
            return bad("truncated list");
          const size_t cnt = static_cast<size_t>(v);
          for (size_t k = 0; k < cnt; ++k)
            if (!next_token(p, end, ts, te) || !parse_token(ts, te, pr.type, v, raw)) return bad("truncated list data");
          continue;
        }
        if (!next_token(p, end, ts, te) || !parse_token(ts, te, pr.type, v, raw))
          return bad("truncated or malformed " + e.name + " data");
        if (isv) assign(pt, pr.field, pr.type, v, raw);
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
    std::vector<unsigned char> buf(n * 31);  // memory-bound: one thread
    for (size_t i = 0; i < n; ++i) {
      unsigned char* o = &buf[i * 31];
      const lcr_point& q = pts[i];
      std::memcpy(o, &q.x, 4);
      std::memcpy(o + 4, &q.y, 4);
      std::memcpy(o + 8, &q.z, 4);
      o[12] = q.r;
      o[13] = q.g;
      o[14] = q.b;
      std::memcpy(o + 15, &q.normal_x, 4);
      std::memcpy(o + 19, &q.normal_y, 4);
      std::memcpy(o + 23, &q.normal_z, 4);
      std::memcpy(o + 27, &q.curvature, 4);
    }
    ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  } else {
    // shortest text that reads back to the same float (to_chars), formatted in parallel
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t parts = n >= 65536 ? hw : 1;
    std::vector<std::string> chunk(parts);
    parallel_ranges(n, [&](size_t b, size_t en, size_t k) {
      std::string& s = chunk[parts == 1 ? 0 : k];
      s.reserve((en - b) * 96);
      char tmp[64];
      auto put_f = [&](float v, char sep) {
        const auto r = std::to_chars(tmp, tmp + sizeof tmp, v);
        s.append(tmp, r.ptr);
        s.push_back(sep);
      };
      auto put_u = [&](unsigned v, char sep) {
        const auto r = std::to_chars(tmp, tmp + sizeof tmp, v);
        s.append(tmp, r.ptr);
        s.push_back(sep);
      };
      for (size_t i = b; i < en; ++i) {
        const lcr_point& q = pts[i];
        put_f(q.x, ' ');
        put_f(q.y, ' ');
        put_f(q.z, ' ');
        put_u(q.r, ' ');
        put_u(q.g, ' ');
        put_u(q.b, ' ');
        put_f(q.normal_x, ' ');
        put_f(q.normal_y, ' ');
        put_f(q.normal_z, ' ');
        put_f(q.curvature, '\n');
      }
      return true;
    });
    for (const std::string& s : chunk)
      if (ok && !s.empty()) ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? LCR_OK : fail(LCR_ERR_IO, std::string("write failed: ") + path);
}

}  // extern "C"
