// Dependency-free command-line handling for the tools: the option names,
// short aliases, defaults and help layout of boost::program_options as the
// reference tools declare them, plus PLY load/save and PCL-style cloud dumps.
#pragma once

#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "lcr_pcl.hpp"

namespace cli {

// Raised for unknown options / missing values (boost::program_options::error).
class OptionError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

class Options {
 public:
  explicit Options(const char* caption) : caption_(caption) {}
  // spec "long,s" or "long"; has_value=false declares a switch.
  Options& add(const char* spec, bool has_value, const char* def, const char* help);
  void parse(int argc, char** argv);
  bool count(const std::string& name) const;
  std::string str(const std::string& name) const;
  double num(const std::string& name) const;
  long integer(const std::string& name) const;
  void print(std::ostream& os) const;

 private:
  struct Opt {
    std::string name;
    char shrt = 0;
    bool has_value = false;
    bool has_default = false;
    std::string def, help, value;
    bool seen = false;
  };
  const Opt* find(const std::string& name) const;
  Opt* find_long(const std::string& name);
  Opt* find_short(char c);
  std::string caption_;
  std::vector<Opt> opts_;
};

lcr::PointCloud::Ptr load_cloud(const std::string& path);
void save_cloud(const std::string& path, const lcr::PointCloud& c);
// What `std::cout << *cloud` prints for a pcl::PointCloud.
void print_cloud(std::ostream& os, const lcr::PointCloud& c);
// What `std::cout << Eigen::Matrix4f` prints (aligned columns, stream precision).
void print_matrix(std::ostream& os, const lcr::Matrix4f& m);
// Strips a trailing ".ply" and appends suffix (outlier_removal.cpp:94-96).
std::string with_suffix(std::string name, const std::string& suffix);

}  // namespace cli
