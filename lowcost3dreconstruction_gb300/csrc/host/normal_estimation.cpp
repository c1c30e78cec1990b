// normal_estimation: NormalEstimation, a drop-in for pcl_tools/normal_estimation.cpp.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("neighbors,n", true, "50", "N. of neighbors to analyze for each point")
        .add("reverse_normals,r", false, nullptr, "Reverse normals' direction")
        .add("centroid,c", false, nullptr, "Use the centroid as defined view point")
        .add("origin,z", false, nullptr, "Use the origin as defined view point");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Estimate a set of normals for all the points in the input dataset." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i input.ply -o output.ply [opts]");
    const long k = desc.integer("neighbors");
    if (k <= 0) throw std::runtime_error("neighbors must be positive");
    const bool reverse = desc.count("reverse_normals"), centroid = desc.count("centroid"),
               origin = desc.count("origin");
    if (origin && centroid)
      throw std::runtime_error("It is not possible to use the centroid and origin as viewpoint at the same time");
    const std::string in = desc.str("input"), out = desc.str("output");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    lcr::NormalEstimation ne;
    ne.setInputCloud(cloud);
    ne.setKSearch(static_cast<int>(k));
    if (centroid) {
      std::array<float, 4> c;
      lcr::compute3DCentroid(*cloud, c);
      ne.setViewPoint(c[0], c[1], c[2]);
    } else if (origin) {
      ne.useSensorOriginAsViewPoint();
    }
    // With the centroid as viewpoint normals point inwards; flip them outwards
    // unless reversed (normal_estimation.cpp:112-118).
    lcr::PointCloud result;
    ne.compute(result, (centroid && !reverse) || (!centroid && reverse));
    cli::save_cloud(out, result);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
