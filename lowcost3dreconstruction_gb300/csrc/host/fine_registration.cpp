// fine_registration: pairwise ICP, a drop-in for pcl_tools/fine_registration.cpp
// (same flags, defaults, messages and exit codes).  --point_to_plane is an
// addition (point-to-plane error; needs target normals).
#include <iostream>

#include "cli_common.h"

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Input cloud file (.ply)")
        .add("target,t", true, nullptr, "Input target file (.ply)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("accumulated,a", true, nullptr, "Save the accumulated point cloud")
        .add("distance_threshold", true, "0.1", "The maximum distance threshold between two correspondent points")
        .add("max_iterations", true, "50", "The maximum number of iterations the internal optimization should run for")
        .add("transformation_epsilon", true, "1e-09",
             "Maximum allowable difference between two consecutive transformations to be considered as having converged")
        .add("euclidean_fitness_epsilon", true, "0.001",
             "Maximum allowed Euclidean error between two consecutive steps in the ICP loop, before the algorithm is "
             "considered to have converged")
        .add("point_to_plane", false, nullptr, "Minimise the point-to-plane error (uses target normals)");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("target") && desc.count("output")))
      throw std::string("Correct mode of use: " + std::string(argv[0]) +
                        " -i input.ply -t target.ply -o output.ply [opts]");
    const long max_iterations = desc.integer("max_iterations");
    if (max_iterations <= 0) throw std::string("max_iterations needs to be greater than zero.");
    const double distance_threshold = desc.num("distance_threshold");
    const double transformation_epsilon = desc.num("transformation_epsilon");
    const double euclidean_fitness_epsilon = desc.num("euclidean_fitness_epsilon");
    const std::string src_file = desc.str("input"), tgt_file = desc.str("target"), out_file = desc.str("output");

    lcr::PointCloud::Ptr src = cli::load_cloud(src_file);
    if (!src) throw std::string("Couldn't load input cloud file");
    std::cout << "Loaded " << src->size() << " data points from " << src_file << std::endl;
    lcr::PointCloud::Ptr tgt = cli::load_cloud(tgt_file);
    if (!tgt) throw std::string("Couldn't load input target file");
    std::cout << "Loaded " << tgt->size() << " data points from " << tgt_file << std::endl;

    lcr::IterativeClosestPoint icp;
    icp.setInputSource(src);
    icp.setInputTarget(tgt);
    icp.setMaxCorrespondenceDistance(distance_threshold);
    icp.setMaximumIterations(static_cast<int>(max_iterations));
    icp.setTransformationEpsilon(transformation_epsilon);
    icp.setEuclideanFitnessEpsilon(euclidean_fitness_epsilon);
    icp.setPointToPlane(desc.count("point_to_plane"));
    lcr::PointCloud registered;
    icp.align(registered);

    const lcr::Matrix4f T = icp.getFinalTransformation();
    std::cout << "Has converged: " << (icp.hasConverged() ? "True" : "False") << std::endl
              << "Score: " << icp.getFitnessScore() << std::endl;
    cli::print_matrix(std::cout, T);
    std::cout << std::endl;
    cli::save_cloud(out_file, registered);
    if (desc.count("accumulated")) cli::save_cloud(desc.str("accumulated"), registered + *tgt);
    return 0;
  } catch (const cli::OptionError& e) {
    std::cerr << "ERROR: " << e.what() << std::endl;
  } catch (const std::string& msg) {
    std::cerr << msg << std::endl;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  }
  return -1;
}
