// transform: apply a 4x4 matrix read from a text file to points and normals, a
// drop-in for pcl_tools/transform.cpp.
#include <fstream>
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("transform,t", true, nullptr, "Transform matrix file (.txt)");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Apply a rigid transformation to a point cloud." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output") && desc.count("transform")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) +
                             " -i input.ply -o output.ply -t transform_file.txt");
    const std::string in = desc.str("input"), out = desc.str("output"), tf = desc.str("transform");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    std::ifstream file(tf);
    if (!file.is_open()) throw std::runtime_error("Unable to open file: " + tf);
    lcr::Matrix4f T;
    for (int i = 0; i < 16; ++i) {
      double v;
      if (!(file >> v)) throw std::runtime_error("Error on read transform file: " + tf);
      T.m[i] = static_cast<float>(v);
    }
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
