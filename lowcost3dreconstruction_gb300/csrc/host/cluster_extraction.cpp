// cluster_extraction: Euclidean cluster extraction, a drop-in for
// pcl_tools/cluster_extraction.cpp (options :41-67, clusters :84-104,
// extraction :106-130).  Clusters hold at least n * cluster_percentage points
// (the product truncated to an integer, as setMinClusterSize(int) receives it)
// and at most n; the output holds the clusters' points, largest cluster first,
// ascending input order within each; --outliers_file writes the rest.
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("outliers_file,f", false, nullptr, "Saves the removed points in a .ply file")
        .add("cluster_percentage,p", true, "0.25",
             "Percentage (0 to 1) of points that a cluster needs to contain in order to be considered valid")
        .add("tolerance,t", true, "0.02", "Spatial cluster tolerance as a measure in the L2 Euclidean space");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Euclidean cluster extraction." << std::endl << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i input.ply -o output.ply");
    const double pct = desc.num("cluster_percentage"), tol = desc.num("tolerance");
    if (pct < 0 || pct > 1) throw std::logic_error("cluster_percentage must be a value between 0 and 1");
    const std::string in = desc.str("input"), out = desc.str("output");
    lcr::PointCloud::Ptr cloud = cli::load_cloud(in);
    if (!cloud) throw std::runtime_error("Couldn't load input point cloud: " + in);
    std::cout << "Cloud before filtering: " << std::endl;
    cli::print_cloud(std::cout, *cloud);
    std::cout << std::endl;
    lcr::Context& ctx = lcr::Context::thread_default();
    lcr::DeviceCloud d(ctx, *cloud);
    const size_t n = cloud->size();
    const size_t min_size = static_cast<size_t>(static_cast<int>(static_cast<double>(n) * pct));
    size_t k = 0;
    lcr_cloud *kept = nullptr, *rest = nullptr;
    ctx.check(lcr_euclidean_clusters(ctx.get(), d.get(), tol, min_size, n, nullptr, &k, &kept, &rest));
    lcr::DeviceCloud dk(ctx, kept), dr(ctx, rest);
    if (k == 0) throw std::runtime_error("Could not extact clusters for the given dataset");
    std::cout << k << " cluster(s) extracted." << std::endl << std::endl;
    lcr::PointCloud clustered, outliers;
    dk.download(clustered);
    std::cout << "Cloud after filtering: " << std::endl;
    cli::print_cloud(std::cout, clustered);
    std::cout << std::endl;
    cli::save_cloud(out, clustered);
    if (desc.count("outliers_file")) {
      dr.download(outliers);
      cli::save_cloud(cli::with_suffix(out, "_outliers.ply"), outliers);
    }
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
