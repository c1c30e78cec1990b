#include "cli_common.h"

#include <algorithm>
#include <cstdlib>
#include <iomanip>
#include <sstream>

namespace cli {

Options& Options::add(const char* spec, bool has_value, const char* def, const char* help) {
  Opt o;
  std::string s(spec);
  const size_t c = s.find(',');
  o.name = s.substr(0, c);
  if (c != std::string::npos && c + 1 < s.size()) o.shrt = s[c + 1];
  o.has_value = has_value;
  o.has_default = def != nullptr;
  if (def) o.def = def;
  o.help = help;
  opts_.push_back(o);
  return *this;
}

Options::Opt* Options::find_long(const std::string& n) {
  for (Opt& o : opts_)
    if (o.name == n) return &o;
  return nullptr;
}

Options::Opt* Options::find_short(char ch) {
  for (Opt& o : opts_)
    if (o.shrt == ch) return &o;
  return nullptr;
}

const Options::Opt* Options::find(const std::string& n) const {
  for (const Opt& o : opts_)
    if (o.name == n) return &o;
  return nullptr;
}

void Options::parse(int argc, char** argv) {
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    Opt* o = nullptr;
    std::string inline_val;
    bool has_inline = false;
    if (a.rfind("--", 0) == 0) {
      std::string n = a.substr(2);
      const size_t eq = n.find('=');
      if (eq != std::string::npos) {
        inline_val = n.substr(eq + 1);
        n = n.substr(0, eq);
        has_inline = true;
      }
      o = find_long(n);
      if (!o) throw OptionError("unrecognised option '" + a + "'");
    } else if (a.size() >= 2 && a[0] == '-') {
      o = find_short(a[1]);
      if (!o) throw OptionError("unrecognised option '" + a.substr(0, 2) + "'");
      if (a.size() > 2) {
        inline_val = a.substr(2);
        has_inline = true;
      }
    } else {
      throw OptionError("too many positional options have been specified on the command line");
    }
    if (o->has_value) {
      if (has_inline) {
        o->value = inline_val;
      } else {
        if (i + 1 >= argc) throw OptionError("the required argument for option '--" + o->name + "' is missing");
        o->value = argv[++i];
      }
    } else if (has_inline) {
      throw OptionError("option '--" + o->name + "' does not take any arguments");
    }
    o->seen = true;
  }
}

bool Options::count(const std::string& n) const {
  const Opt* o = find(n);
  return o && (o->seen || (o->has_value && o->has_default));
}

std::string Options::str(const std::string& n) const {
  const Opt* o = find(n);
  if (!o) throw std::logic_error("unknown option " + n);
  return o->seen ? o->value : o->def;
}

double Options::num(const std::string& n) const {
  const std::string v = str(n);
  char* end = nullptr;
  const double d = std::strtod(v.c_str(), &end);
  if (v.empty() || !end || *end) throw OptionError("the argument ('" + v + "') for option '--" + n + "' is invalid");
  return d;
}

long Options::integer(const std::string& n) const {
  const std::string v = str(n);
  char* end = nullptr;
  const long d = std::strtol(v.c_str(), &end, 10);
  if (v.empty() || !end || *end) throw OptionError("the argument ('" + v + "') for option '--" + n + "' is invalid");
  return d;
}

void Options::print(std::ostream& os) const {
  os << caption_ << ":\n";
  for (const Opt& o : opts_) {
    std::string left = "  ";
    if (o.shrt) left += std::string("-") + o.shrt + " [ --" + o.name + " ]";
    else left += "--" + o.name;
    if (o.has_value) left += o.has_default ? " arg (=" + o.def + ")" : " arg";
    if (left.size() < 40) left += std::string(40 - left.size(), ' ');
    else left += " ";
    os << left << o.help << "\n";
  }
}

lcr::PointCloud::Ptr load_cloud(const std::string& path) {
  auto c = std::make_shared<lcr::PointCloud>();
  if (lcr::io::loadPLYFile(path, *c) == -1) return nullptr;
  return c;
}

void save_cloud(const std::string& path, const lcr::PointCloud& c) {
  if (lcr::io::savePLYFileBinary(path, c) != 0) throw std::runtime_error("Couldn't write point cloud: " + path);
}

void print_cloud(std::ostream& os, const lcr::PointCloud& c) {
  os << "header: seq: 0 stamp: 0 frame_id: \n\n"
     << "points[]: " << c.size() << "\n"
     << "width: " << c.size() << "\n"
     << "height: 1\n"
     << "is_dense: 1\n"
     << "sensor origin (xyz): [0, 0, 0] / orientation (xyzw): [0, 0, 0, 1]\n";
}

void print_matrix(std::ostream& os, const lcr::Matrix4f& m) {
  std::string cell[16];
  size_t w = 0;
  for (int i = 0; i < 16; ++i) {
    std::ostringstream s;
    s.precision(os.precision());
    s << m.m[i];
    cell[i] = s.str();
    w = std::max(w, cell[i].size());
  }
  for (int r = 0; r < 4; ++r) {
    for (int c = 0; c < 4; ++c) {
      if (c) os << ' ';
      os << std::setw(static_cast<int>(w)) << cell[4 * r + c];
    }
    if (r < 3) os << '\n';
  }
}

std::string with_suffix(std::string name, const std::string& suffix) {
  const size_t pos = name.rfind(".ply");
  if (pos != std::string::npos) name.erase(pos, 4);
  return name + suffix;
}

}  // namespace cli
