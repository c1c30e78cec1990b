// accumulate_clouds: a drop-in for pcl_tools/accumulate_clouds.cpp -- target plus
// the source points that no target point's cube [q-r, q+r] contains, cleaned by
// SOR; --all skips the crop and the cleaning; --negative also saves the
// remaining source points.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input cloud file (.ply)")
        .add("target,t", true, nullptr, "Input target file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("radius,r", true, "0.05", "Standard radius to select point neighbours")
        .add("clean_neighbors,c", true, "50", "N. of neighbors to analyze for each point to clean")
        .add("dev_mult,d", true, "1", "Standard deviation multiplier to clean")
        .add("negative,n", false, nullptr, "Saves the not redundant points in a .ply file")
        .add("all,a", false, nullptr, "Saves accumulated cloud with all points in a .ply file");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Accumulate points clouds removing redundant points" << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("target") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) +
                             " -i input.ply -t target.ply -o output.ply [opts]");
    const long k = desc.integer("clean_neighbors");
    if (k <= 0) throw std::runtime_error("clean_neighbors must be positive");
    const double mul = desc.num("dev_mult"), radius = desc.num("radius");
    const std::string src_file = desc.str("input"), tgt_file = desc.str("target");
    std::string out_file = desc.str("output");
    lcr::PointCloud::Ptr src = cli::load_cloud(src_file);
    if (!src) throw std::runtime_error("Couldn't load input point cloud: " + src_file);
    std::cout << "Loaded " << src->size() << " data points from " << src_file << std::endl;
    lcr::PointCloud::Ptr tgt = cli::load_cloud(tgt_file);
    if (!tgt) throw std::runtime_error("Couldn't load target point cloud: " + tgt_file);
    std::cout << "Loaded " << tgt->size() << " data points from " << tgt_file << std::endl;
    std::cout << "Cloud before accumulate: " << std::endl;
    cli::print_cloud(std::cout, *tgt);
    std::cout << std::endl;

    lcr::Context& ctx = lcr::Context::thread_default();
    lcr::DeviceCloud ds(ctx, *src), dt(ctx, *tgt);
    lcr_cloud *out = nullptr, *rem = nullptr;
    ctx.check(lcr_accumulate(ctx.get(), ds.get(), dt.get(), radius, static_cast<int>(k), mul,
                             desc.count("all") ? LCR_ACCUM_ALL : 0, &out, &rem));
    lcr::PointCloud accumulated, remaining;
    lcr::DeviceCloud(ctx, out).download(accumulated);
    lcr::DeviceCloud(ctx, rem).download(remaining);
    std::cout << "Cloud after accumulate: " << std::endl;
    cli::print_cloud(std::cout, accumulated);
    std::cout << std::endl;
    cli::save_cloud(out_file, accumulated);
    if (desc.count("negative")) cli::save_cloud(cli::with_suffix(out_file, "_negative.ply"), remaining);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
