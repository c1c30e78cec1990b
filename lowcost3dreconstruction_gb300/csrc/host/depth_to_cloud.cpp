// depth_to_cloud: burst fusion + back-projection of depth frames to a PLY cloud,
// the arithmetic of capture/depth_capture/depth_capture.cpp:save_ply (Kinect v1,
// uint16 mm), capture/super_resolution/super_resolution.cpp:295-309 (zero-
// eliminated mean over a burst) and capture/depth_capture_kv2 (Kinect v2, float
// mm).  Frames are read from raw files (row-major, little-endian uint16 or
// float32) or 16-bit binary PGM; the device capture and PNG/OpenCV front ends of
// the reference are not part of this tool.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <vector>

#include "cli_common.h"

namespace {

std::vector<char> read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("Image can not be read: " + path);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// 16-bit binary PGM (P5, maxval > 255, big-endian samples) -> uint16 row-major.
bool read_pgm16(const std::vector<char>& buf, int& w, int& h, std::vector<uint16_t>& out) {
  if (buf.size() < 2 || buf[0] != 'P' || buf[1] != '5') return false;
  std::string hdr(buf.begin(), buf.begin() + std::min<size_t>(buf.size(), 512));
  std::istringstream s(hdr.substr(2));
  int maxv = 0;
  s >> w >> h >> maxv;
  if (!s || w <= 0 || h <= 0 || maxv <= 255) return false;
  const size_t off = static_cast<size_t>(s.tellg()) + 2 + 1;
  if (buf.size() < off + static_cast<size_t>(w) * h * 2) return false;
  out.resize(static_cast<size_t>(w) * h);
  for (size_t i = 0; i < out.size(); ++i)
    out[i] = static_cast<uint16_t>((static_cast<unsigned char>(buf[off + 2 * i]) << 8) |
                                   static_cast<unsigned char>(buf[off + 2 * i + 1]));
  return true;
}

}  // namespace

int main(int argc, char* argv[]) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "Depth frame(s): comma-separated .raw/.pgm files (a burst is fused)")
        .add("output,o", true, nullptr, "Output file (.ply)")
        .add("kinect_version,k", true, "1", "1: uint16 mm frames (Kinect v1), 2: float32 mm frames (Kinect v2)")
        .add("width,W", true, "640", "Frame width")
        .add("height,H", true, "480", "Frame height")
        .add("fx", true, "572.882768", "Focal length x")
        .add("fy", true, "542.73998", "Focal length y")
        .add("cx", true, "314.649173", "Principal point x")
        .add("cy", true, "240.160459", "Principal point y")
        .add("depth_min,m", true, "0", "Minimum value for depth (threshold)")
        .add("depth_max,M", true, "65535", "Maximum value for depth (threshold)")
        .add("left_plane,l", true, "0", "Left plane threshold (pixels)")
        .add("right_plane,r", true, "-1", "Right plane threshold (pixels, -1: width-1)")
        .add("top_plane,t", true, "0", "Top plane threshold (pixels)")
        .add("bottom_plane,b", true, "-1", "Bottom plane threshold (pixels, -1: height-1)")
        .add("scale,s", true, "1", "Output units per millimetre")
        .add("no_normals", false, nullptr, "Do not compute image-gradient normals (v1)");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Back-project depth frames (a burst is fused by the zero-eliminated mean) to a point cloud."
                << std::endl
                << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (!(desc.count("input") && desc.count("output")))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i frame0.pgm[,frame1.pgm...] -o out.ply");
    lcr_depth_params p;
    std::memset(&p, 0, sizeof(p));
    p.model = desc.integer("kinect_version") == 2 ? LCR_DEPTH_KINECT_V2 : LCR_DEPTH_KINECT_V1;
    p.width = static_cast<int>(desc.integer("width"));
    p.height = static_cast<int>(desc.integer("height"));
    p.fx = desc.num("fx");
    p.fy = desc.num("fy");
    p.cx = desc.num("cx");
    p.cy = desc.num("cy");
    p.depth_min = desc.num("depth_min");
    p.depth_max = desc.num("depth_max");
    p.scale = desc.num("scale");
    p.normals = desc.count("no_normals") ? 0 : 1;
    p.r = p.g = p.b = 128;
    std::vector<std::string> files;
    std::stringstream ss(desc.str("input"));
    for (std::string f; std::getline(ss, f, ',');)
      if (!f.empty()) files.push_back(f);
    const size_t esz = p.model == LCR_DEPTH_KINECT_V1 ? 2 : 4;
    std::vector<char> frames;
    for (const std::string& f : files) {
      std::vector<char> buf = read_file(f);
      std::vector<uint16_t> pgm;
      int w = 0, h = 0;
      if (p.model == LCR_DEPTH_KINECT_V1 && read_pgm16(buf, w, h, pgm)) {
        p.width = w;
        p.height = h;
        buf.assign(reinterpret_cast<char*>(pgm.data()), reinterpret_cast<char*>(pgm.data() + pgm.size()));
      }
      if (buf.size() != static_cast<size_t>(p.width) * p.height * esz)
        throw std::runtime_error("Unexpected frame size in " + f);
      frames.insert(frames.end(), buf.begin(), buf.end());
    }
    p.frames = static_cast<int>(files.size());
    p.roi_left = static_cast<int>(desc.integer("left_plane"));
    p.roi_top = static_cast<int>(desc.integer("top_plane"));
    const long r = desc.integer("right_plane"), b = desc.integer("bottom_plane");
    p.roi_right = r < 0 ? p.width - 1 : static_cast<int>(r);
    p.roi_bottom = b < 0 ? p.height - 1 : static_cast<int>(b);
    lcr::Context& ctx = lcr::Context::thread_default();
    lcr_cloud* c = nullptr;
    ctx.check(lcr_backproject(ctx.get(), frames.data(), &p, &c));
    lcr::PointCloud cloud;
    lcr::DeviceCloud(ctx, c).download(cloud);
    cli::save_cloud(desc.str("output"), cloud);
    std::cout << desc.str("output") << " saved!" << std::endl;
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
