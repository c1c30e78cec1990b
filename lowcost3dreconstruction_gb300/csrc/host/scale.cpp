// scale: uniform scale of points and normals (matrix diag(s, s, s, 1)), a
// drop-in for pcl_tools/scale.cpp.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("scale,s", true, "1", "Scale factor");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Scale a point cloud." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i input.ply -o output.ply -s [scale]");
    const std::string in = desc.str("input"), out = desc.str("output");
    const float s = static_cast<float>(desc.num("scale"));
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    lcr::Matrix4f T = lcr::Matrix4f::Identity();
    T(0, 0) = T(1, 1) = T(2, 2) = s;
    lcr::PointCloud result;
    lcr::transformPointCloudWithNormals(*cloud, result, T);
    cli::save_cloud(out, result);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
