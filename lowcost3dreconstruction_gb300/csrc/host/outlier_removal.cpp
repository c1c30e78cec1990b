// outlier_removal: StatisticalOutlierRemoval, a drop-in for pcl_tools/outlier_removal.cpp.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("outliers_file,f", false, nullptr, "Saves the outliers in a ply file")
        .add("neighbors,n", true, "50", "Neighbors to analyze for each point")
        .add("dev_mult,d", true, "1", "Standard deviation multiplier");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Remove noisy measurements from a point cloud dataset using statistical analysis techniques."
                << std::endl
                << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i input.ply -o output.ply [opts]");
    const long k = desc.integer("neighbors");
    if (k <= 0) throw std::runtime_error("neighbors must be positive");
    const double mul = desc.num("dev_mult");
    const std::string in = desc.str("input"), out = desc.str("output");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    std::cout << "Cloud before filtering: " << std::endl;
    cli::print_cloud(std::cout, *cloud);
    std::cout << std::endl;
    lcr::StatisticalOutlierRemoval sor;
    sor.setInputCloud(cloud);
    sor.setMeanK(static_cast<int>(k));
    sor.setStddevMulThresh(mul);
    lcr::PointCloud filtered;
    sor.filter(filtered);
    std::cout << "Cloud after filtering: " << std::endl;
    cli::print_cloud(std::cout, filtered);
    std::cout << std::endl;
    cli::save_cloud(out, filtered);
    if (desc.count("outliers_file")) {
      sor.setNegative(true);
      sor.filter(filtered);
      cli::save_cloud(cli::with_suffix(out, "_outliers.ply"), filtered);
    }
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
