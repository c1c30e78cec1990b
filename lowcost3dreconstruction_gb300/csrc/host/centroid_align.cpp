// centroid_align: initial guess by centroids and a roll/pitch/yaw rotation, a
// drop-in for pcl_tools/centroid_align.cpp.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input cloud file (.ply)")
        .add("target,t", true, nullptr, "Input target file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("accumulated,a", true, nullptr, "Saves the accumulated cloud in a .ply file")
        .add("roll,r", true, "0", "Rotation in X - degrees (Roll)")
        .add("pitch,p", true, "0", "Rotation in Y - degrees (Pitch)")
        .add("yaw,y", true, "0", "Rotation in Z - degrees (Yaw)")
        .add("elevation,e", true, "0", "Translation in Y");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Align the centroids of two point clouds." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("target") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) +
                             " -i input.ply -t target.ply -o output.ply [opts]");
    const std::string src_file = desc.str("input"), tgt_file = desc.str("target"), out_file = desc.str("output");
    lcr::PointCloud::Ptr src = cli::load_cloud(src_file);
    if (!src) throw std::runtime_error("Couldn't load input point cloud: " + src_file);
    std::cout << "Loaded " << src->size() << " data points from " << src_file << std::endl;
    lcr::PointCloud::Ptr tgt = cli::load_cloud(tgt_file);
    if (!tgt) throw std::runtime_error("Couldn't load target point cloud: " + tgt_file);
    std::cout << "Loaded " << tgt->size() << " data points from " << tgt_file << std::endl;
    lcr::Context& ctx = lcr::Context::thread_default();
    lcr::DeviceCloud ds(ctx, *src), dt(ctx, *tgt);
    lcr_cloud* out = nullptr;
    float m[16];
    ctx.check(lcr_centroid_align(ctx.get(), ds.get(), dt.get(), desc.num("roll"), desc.num("pitch"), desc.num("yaw"),
                                 desc.num("elevation"), &out, m));
    lcr::PointCloud moved;
    lcr::DeviceCloud(ctx, out).download(moved);
    cli::save_cloud(out_file, moved);
    if (desc.count("accumulated")) cli::save_cloud(desc.str("accumulated"), moved + *tgt);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
