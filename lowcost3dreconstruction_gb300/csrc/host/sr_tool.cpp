// The super-resolution tools: each view's depth burst fused into one depth
// image and cloud.  kv2 = false is capture/super_resolution/
// super_resolution.cpp (options :142-211, per view :212-320): 16-bit PNG
// frames, a 16-bit fused PNG.  kv2 = true is capture/super_resolution_kv2/
// super_resolution_kv2.cpp (the same options and messages): float frames
// stored as 8-bit RGBA PNGs, a float fused image stored the same way, its
// cloud through the float pinhole model.  Per view: read
// <name>_burst_<view>_<i>.png (i < sr_size), register, warp, upsample, fuse
// and resample on the GPU (lcr_super_resolve / lcr_super_resolve_f32), write
// <name>_srdepth_<view>.png and <name>_srmesh_<view>.ply (the points with
// depth inside the burst's observed range, image-gradient normals, colour
// 128, millimetres, ASCII as save_ply writes).
#include "sr_tool.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <thread>
#include <vector>

#include "cli_common.h"
#include "png16.h"

namespace sr_tool {

int run(int argc, char* argv[], bool kv2) {
  try {
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("capture_name,n", true, "artefact", "Prefix of saved files")
        .add("capture_step,s", true, "20", "Angles (in degrees) for each capture")
        .add("num_captures,c", true, "18", "Number of view points (anlges)")
        .add("sr_size,z", true, "16", "Number of sr images for each capture")
        .add("resample_factor,f", true, "4", "Resample factor")
        .add("view_angle,a", true, nullptr, "Make SR just for an unique view angle")
        .add("top,t", false, nullptr, "Make SR for top view")
        .add("bottom,b", false, nullptr, "Make SR for bottom view");
    desc.parse(argc, argv);
    if (desc.count("help")) {
      std::cout << "Super-resolution tool to reconstruct detail and obtain high-resolution "
                << "depth images from the acquired image bursts." << std::endl
                << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    const std::string name = desc.str("capture_name");
    long step = desc.integer("capture_step"), ncap = desc.integer("num_captures");
    const long sr_size = desc.integer("sr_size"), factor = desc.integer("resample_factor");
    const int picks = static_cast<int>(desc.count("view_angle")) + static_cast<int>(desc.count("top")) +
                      static_cast<int>(desc.count("bottom"));
    // Option rules, checked in this order.  A rule that holds prints its
    // message; kStop ends the tool with -1 (message on stdout, as the capture
    // tools print it), kError throws (stderr), kNote only informs.
    enum Action { kStop, kError, kNote };
    struct Rule {
      bool holds;
      Action action;
      const char* message;
    };
    const Rule rules[] = {
        {factor <= 0, kStop, "The command option 'resample_factor', must be bigger than zero"},
        {sr_size <= 0, kError, "sr_size must be positive"},
        {step < 0 || ncap < 0, kError, "capture_step and num_captures must not be negative"},
        {picks > 1, kStop,
         "The command options: 'view_angle', 'top' and 'bottom' can not be used together. Choose only one of them"},
        {picks == 1, kNote,
         "When using the command options: 'view_angle', 'top' or 'bottom', the options 'capture_step' and "
         "'num_captures' are ignored"},
    };
    for (const Rule& r : rules) {
      if (!r.holds) continue;
      if (r.action == kError) throw std::logic_error(r.message);
      std::cout << r.message << std::endl;
      if (r.action == kStop) return -1;
    }
    const bool single = picks == 1;
    std::string view;
    if (single) {
      step = 0;
      ncap = 1;
      view = desc.count("view_angle") ? std::to_string(desc.integer("view_angle") % 360)
                                      : (desc.count("top") ? "top" : "bottom");
    }
    std::cout << "Capture name: " << name << std::endl;
    if (single) {
      std::cout << "View angle: " << view << std::endl;
    } else {
      std::cout << "Step: " << step << std::endl;
      std::cout << "N. of captures: " << ncap << std::endl;
    }
    std::cout << std::endl;
    for (long c = 0; c < ncap; ++c) {
      if (!single) view = std::to_string(c * step);
      std::vector<uint16_t> burst;
      std::vector<float> burst_f;
      int w = 0, h = 0;
      // The frames decode in parallel (PNG inflate and unfiltering are the
      // tool's largest host cost); the first unreadable frame in index order,
      // or one whose size differs from frame 0, is reported.
      struct Frame {
        std::vector<uint16_t> px;
        std::vector<float> pf;
        int w = 0, h = 0;
        bool ok = false;
      };
      std::vector<Frame> fr(static_cast<size_t>(sr_size));
      auto file_of = [&](long i) { return name + "_burst_" + view + "_" + std::to_string(i) + ".png"; };
      auto decode = [&](long i) {
        Frame& f = fr[static_cast<size_t>(i)];
        std::string err;
        if (kv2) {
          std::vector<unsigned char> rgba;
          f.ok = png16::read_rgba8(file_of(i), rgba, f.w, f.h, err);
          if (f.ok) {
            // the four bytes of each float, stored by OpenCV as a BGRA pixel
            const size_t n = static_cast<size_t>(f.w) * f.h;
            f.pf.resize(n);
            for (size_t k = 0; k < n; ++k) {
              const unsigned char by[4] = {rgba[4 * k + 2], rgba[4 * k + 1], rgba[4 * k], rgba[4 * k + 3]};
              std::memcpy(&f.pf[k], by, 4);
            }
          }
        } else {
          f.ok = png16::read(file_of(i), f.px, f.w, f.h, err);
        }
      };
      {
        const long nt = std::max(1L, std::min<long>(sr_size, std::thread::hardware_concurrency()));
        std::atomic<long> next{0};
        std::vector<std::thread> pool;
        for (long t = 0; t < nt; ++t)
          pool.emplace_back([&] {
            for (long i; (i = next++) < sr_size;) decode(i);
          });
        for (auto& t : pool) t.join();
      }
      for (long i = 0; i < sr_size; ++i) {
        const Frame& f = fr[static_cast<size_t>(i)];
        if (!f.ok || f.w != fr[0].w || f.h != fr[0].h) {
          std::cout << "Image can not be read: " << file_of(i) << std::endl;
          return -1;
        }
      }
      w = fr[0].w;
      h = fr[0].h;
      const size_t plane = static_cast<size_t>(w) * h;
      if (kv2) {
        burst_f.resize(plane * sr_size);
        for (long i = 0; i < sr_size; ++i) std::copy(fr[i].pf.begin(), fr[i].pf.end(), burst_f.begin() + plane * i);
      } else {
        burst.resize(plane * sr_size);
        for (long i = 0; i < sr_size; ++i) std::copy(fr[i].px.begin(), fr[i].px.end(), burst.begin() + plane * i);
      }
      fr.clear();
      lcr::Context& ctx = lcr::Context::thread_default();
      lcr_sr_params sp;
      sp.width = w;
      sp.height = h;
      sp.frames = static_cast<int>(sr_size);
      sp.factor = static_cast<int>(factor);
      sp.ecc_iterations = 200;
      sp.ecc_epsilon = 1e-12;
      std::vector<uint16_t> fused(kv2 ? 0 : static_cast<size_t>(w) * h);
      std::vector<float> fused_f(kv2 ? static_cast<size_t>(w) * h : 0);
      std::vector<float> warps(6 * sr_size);
      float mm[2];
      if (kv2)
        ctx.check(lcr_super_resolve_f32(ctx.get(), burst_f.data(), &sp, fused_f.data(), warps.data(), mm, nullptr));
      else
        ctx.check(lcr_super_resolve(ctx.get(), burst.data(), &sp, fused.data(), warps.data(), mm, nullptr));
      std::printf("Observed Global Min: %.0lf\n", static_cast<double>(mm[0]));
      std::printf("Observed Global Max: %.0lf\n", static_cast<double>(mm[1]));
      for (long i = 0; i < sr_size; ++i) {
        const float* m = &warps[6 * i];
        std::cout << "View(" << view << ") Alignment " << i << "-> 0 = [" << m[0] << ", " << m[1] << ", " << m[2]
                  << ";\n " << m[3] << ", " << m[4] << ", " << m[5] << "]" << std::endl;
      }
      std::string err;
      const std::string png = name + "_srdepth_" + view + ".png";
      if (kv2) {
        std::vector<unsigned char> rgba(static_cast<size_t>(w) * h * 4);
        for (size_t k = 0; k < fused_f.size(); ++k) {
          unsigned char b[4];
          std::memcpy(b, &fused_f[k], 4);
          rgba[4 * k] = b[2];
          rgba[4 * k + 1] = b[1];
          rgba[4 * k + 2] = b[0];
          rgba[4 * k + 3] = b[3];
        }
        if (!png16::write_rgba8(png, rgba.data(), w, h, err)) throw std::runtime_error(err);
      } else if (!png16::write(png, fused.data(), w, h, err)) {
        throw std::runtime_error(err);
      }
      lcr_depth_params dp{};
      dp.model = kv2 ? LCR_DEPTH_PINHOLE_F32 : LCR_DEPTH_KINECT_V1;
      dp.width = w;
      dp.height = h;
      dp.frames = 1;
      // the intrinsics save_ply uses (super_resolution.cpp:108, super_resolution_kv2.cpp:100)
      dp.fx = kv2 ? 365.531799 : 572.882768;
      dp.fy = kv2 ? 365.531799 : 542.739980;
      dp.cx = kv2 ? 256.136810 : 314.649173;
      dp.cy = kv2 ? 206.013901 : 240.160459;
      dp.depth_min = mm[0];
      dp.depth_max = mm[1];
      dp.roi_left = 0;
      dp.roi_right = w - 1;
      dp.roi_top = 0;
      dp.roi_bottom = h - 1;
      dp.scale = 1.0;
      dp.normals = 1;
      dp.r = dp.g = dp.b = 128;
      lcr_cloud* cl = nullptr;
      const void* fused_px = kv2 ? static_cast<const void*>(fused_f.data()) : fused.data();
      ctx.check(lcr_backproject(ctx.get(), fused_px, &dp, &cl));
      lcr::PointCloud pc;
      lcr::DeviceCloud(ctx, cl).download(pc);
      const std::string ply = name + "_srmesh_" + view + ".ply";
      if (lcr_ply_write(ply.c_str(), pc.points.data(), pc.points.size(), 0) != LCR_OK)
        throw std::runtime_error(lcr_ply_last_error());
      std::printf("%s saved!\n", ply.c_str());
      std::cout << std::endl;
    }
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}

}  // namespace sr_tool
