// cloud_downsampling: VoxelGrid, a drop-in for pcl_tools/cloud_downsampling.cpp.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("leaf_size,s", true, "1", "Leaf size for pcl::VoxelGrid filter in meters");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Reduce the number of points of a point cloud, using a voxelized grid approach." << std::endl
                << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i input.ply -o output.ply [opts]");
    const float leaf = static_cast<float>(desc.num("leaf_size"));
    const std::string in = desc.str("input"), out = desc.str("output");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    std::cout << "Cloud before filtering: " << std::endl;
    cli::print_cloud(std::cout, *cloud);
    std::cout << std::endl;
    lcr::VoxelGrid sor;
    sor.setInputCloud(cloud);
    sor.setLeafSize(leaf, leaf, leaf);
    lcr::PointCloud filtered;
    sor.filter(filtered);
    std::cout << "Cloud after filtering: " << std::endl;
    cli::print_cloud(std::cout, filtered);
    std::cout << std::endl;
    cli::save_cloud(out, filtered);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
