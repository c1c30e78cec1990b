// planar_segmentation: remove the dominant plane, a drop-in for
// pcl_tools/planar_segmentation.cpp (options :41-64, SACSegmentation :74-89,
// extraction :91-110).  RANSAC runs 1024 seeded hypotheses at once on the
// GPU (the reference draws up to 50 with rand()), then refits the best plane
// by least squares and selects its inliers again, as setOptimizeCoefficients
// does.  The output holds the points off the plane; --negative writes the
// plane's points to <output>_plane.ply.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("threshold,t", true, "0.05", "Standard radius to remove")
        .add("negative,n", false, nullptr, "Saves the removed points in a .ply file");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Plane model segmentation." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i input.ply -o output.ply");
    const double threshold = desc.num("threshold");
    const std::string in = desc.str("input"), out = desc.str("output");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    std::cout << "Cloud before filtering: " << std::endl;
    cli::print_cloud(std::cout, *cloud);
    std::cout << std::endl;
    lcr::Context& ctx = lcr::Context::thread_default();
    lcr::DeviceCloud d(ctx, *cloud);
    float coef[4];
    size_t ninl = 0;
    lcr_cloud *plane = nullptr, *rest = nullptr;
    ctx.check(lcr_plane_segment(ctx.get(), d.get(), threshold, 1024, 0, coef, &ninl, &plane, &rest));
    lcr::DeviceCloud dp(ctx, plane), dr(ctx, rest);
    if (ninl == 0) throw std::runtime_error("Could not estimate a planar model for the given dataset");
    lcr::PointCloud off, on;
    dr.download(off);
    std::cout << "Cloud after filtering: " << std::endl;
    cli::print_cloud(std::cout, off);
    std::cout << std::endl;
    cli::save_cloud(out, off);
    if (desc.count("negative")) {
      dp.download(on);
      cli::save_cloud(cli::with_suffix(out, "_plane.ply"), on);
    }
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
