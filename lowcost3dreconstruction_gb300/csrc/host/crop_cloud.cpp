// crop_cloud: keep the points inside the box of half-side `radius` around the
// cloud's centroid, a drop-in for pcl_tools/crop_cloud.cpp (options :36-61,
// compute3DCentroid + CropBox :78-88, --negative :90-96).
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("radius,r", true, nullptr, "Standard radius to remove")
        .add("negative,n", false, nullptr, "Saves the removed points in a .ply file");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Filter all data inside of a box." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output") && desc.count("radius")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) +
                             " -i input.ply -o output.ply -r [radius]");
    std::string out = desc.str("output");
    const std::string in = desc.str("input");
    const double radius = desc.num("radius");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    std::cout << "Cloud before filtering: " << std::endl;
    cli::print_cloud(std::cout, *cloud);
    std::cout << std::endl;
    lcr::Context& ctx = lcr::Context::thread_default();
    lcr::DeviceCloud d(ctx, *cloud);
    float c[4];
    ctx.check(lcr_centroid(ctx.get(), d.get(), c));
    // Vector4f(centroid[i] -+ radius): float centroid, double radius, rounded once
    const float lo[3] = {static_cast<float>(c[0] - radius), static_cast<float>(c[1] - radius),
                         static_cast<float>(c[2] - radius)};
    const float hi[3] = {static_cast<float>(c[0] + radius), static_cast<float>(c[1] + radius),
                         static_cast<float>(c[2] + radius)};
    lcr_cloud *inside = nullptr, *outside = nullptr;
    ctx.check(lcr_crop_box(ctx.get(), d.get(), lo, hi, &inside, &outside));
    lcr::PointCloud kept, removed;
    lcr::DeviceCloud(ctx, inside).download(kept);
    lcr::DeviceCloud(ctx, outside).download(removed);
    std::cout << "Cloud after filtering: " << std::endl;
    cli::print_cloud(std::cout, kept);
    std::cout << std::endl;
    cli::save_cloud(out, kept);
    if (desc.count("negative")) cli::save_cloud(cli::with_suffix(out, "_negative.ply"), removed);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
