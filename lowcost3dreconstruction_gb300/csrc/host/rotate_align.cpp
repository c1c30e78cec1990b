// rotate_align without its viewer: orients the lateral views of a turntable
// capture with regard to the first, a drop-in for the headless path of
// rotate_align/rotate_align.cpp (options :122-171, performOperationWithoutGui
// :175-182).  For capture i (file <capture_name><i*step>.ply) it removes the
// non-finite points (:201), translates by (distance_x, distance_y,
// distance_z) and then rotates by -(i*step + i*1.17) degrees about Y
// (transformPointCloud :224-235, two transformPointCloudWithNormals passes),
// writes <capture_name><i*step>_rotated.ply and, with --accumulated_file, the
// concatenation of all views (saveFiles :81-98).  Like the reference it
// returns 0 after printing parse errors.  --gui (the Qt slider window) is not
// available: there is no display, and the tool says so and returns -1.
#include <cmath>
#include <iostream>

#include "cli_common.h"

namespace {

// PCL's DEG2RAD (pcl_macros.h): a double product with this constant.
constexpr double kDeg2Rad = 0.017453293;

// Eigen::AngleAxisf(angle, UnitY).toRotationMatrix() as Eigen evaluates it in
// float: diagonal (1-c) a_i a_i + c, off-diagonal (1-c) a_i a_j -+ s a_k.
lcr::Matrix4f rotation_y(float angle) {
  const float s = std::sin(angle), c = std::cos(angle);
  const float c1 = 1.0f - c;
  lcr::Matrix4f R = lcr::Matrix4f::Identity();
  R(0, 0) = c;
  R(1, 1) = c1 + c;
  R(2, 2) = c;
  R(0, 2) = s;
  R(2, 0) = -s;
  return R;
}

}  // namespace

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("gui,g", false, nullptr, "Show a user interface to edit the distances")
        .add("accumulated_file,a", true, nullptr, "Saves the accumulated mesh in a .ply file")
        .add("capture_name,n", true, "", "Prefix of saved ply files")
        .add("capture_step,s", true, "20", "Angles (in degrees) for each capture")
        .add("num_captures,c", true, "18", "Number of captures")
        .add("distance_x,x", true, "44.0", "Distance in X from kinect to the center of the table")
        .add("distance_y,y", true, "60.0", "Distance in Y from kinect to the center of the table")
        .add("distance_z,z", true, "632.5", "Distance in Z from kinect to the center of the table");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Semi-automatic rotation tool to orient the lateral views with regard to the first." << std::endl
                << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (desc.count("gui")) {
      std::cerr << "The user interface is not available (no display); run without --gui." << std::endl;
      return -1;
    }
    const std::string name = desc.str("capture_name");
    const long step = desc.integer("capture_step"), n = desc.integer("num_captures");
    if (step < 0 || n < 0) throw std::runtime_error("capture_step and num_captures must be non-negative");
    const double dx = desc.num("distance_x"), dy = desc.num("distance_y"), dz = desc.num("distance_z");
    const bool accumulate = desc.count("accumulated_file");
    std::cout << "Capture name: " << name << std::endl;
    std::cout << "Step: " << step << std::endl;
    std::cout << "N. of captures: " << n << std::endl;
    std::cout << "Save accumulated file: " << (accumulate ? "Yes" : "No") << std::endl;

    lcr::Matrix4f T = lcr::Matrix4f::Identity();
    T(0, 3) = static_cast<float>(dx);
    T(1, 3) = static_cast<float>(dy);
    T(2, 3) = static_cast<float>(dz);
    lcr::PointCloud acc;
    std::vector<lcr::PointCloud> views(static_cast<size_t>(n));
    for (long i = 0; i < n; ++i) {
      const std::string file = name + std::to_string(i * step) + ".ply";
      lcr::PointCloud::Ptr c = cli::load_cloud(file);
      if (!c) {
        std::cout << file << " is not a valid file." << std::endl;
        continue;  // the view stays empty, as in the reference
      }
      std::cout << "MESH " << std::to_string(i * step) << " LOADED ALRIGHT!" << std::endl;
      lcr::PointCloud finite, moved;
      lcr::removeNaNFromPointCloud(*c, finite);
      lcr::transformPointCloudWithNormals(finite, moved, T);
      const float angle = static_cast<float>(-((static_cast<double>(i * step) + i * 1.17) * kDeg2Rad));
      lcr::transformPointCloudWithNormals(moved, views[static_cast<size_t>(i)], rotation_y(angle));
    }
    for (long i = 0; i < n; ++i) {
      cli::save_cloud(name + std::to_string(i * step) + "_rotated.ply", views[static_cast<size_t>(i)]);
      if (accumulate) acc += views[static_cast<size_t>(i)];
    }
    if (accumulate) cli::save_cloud(desc.str("accumulated_file"), acc);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return 0;
}
