// pose_proposal: the learned coarse alignment of one pair of captures, a
// drop-in for the Super4PCS call of the coarse stage (scripts/alignment.sh
// :106-113: `Super4PCS -i P.ply Q.ply -r Q_registered.ply -m matrix.txt ...`,
// then `sed -i '1,2d'` on the matrix file and `transform -t` with it).
//
// It proposes the transform taking Q onto P with the shared-MLP pose network
// (lcr_posenet_propose), refines it with point-to-plane ICP (a 2 cm then a
// 1 cm correspondence threshold, in metres) unless --refine 0, and falls back
// to ICP from centroid alignment when the refined proposal does not settle
// (not converged, or inlier RMS above 4 mm).  The matrix file has two header
// lines, which the script deletes, then the 4x4 matrix in the input units.
// --units gives metres per input unit (the script's clouds are scaled by
// 0.01 from millimetres: --units 0.1).  Super4PCS's own tuning options
// (-t -o -d -n) are accepted and ignored.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "cli_common.h"

namespace {

// Reads a little-endian float32 .npy vector of n values.
std::vector<float> load_npy_f32(const std::string& path, size_t n) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("Couldn't open weights file: " + path);
  char magic[8];
  f.read(magic, 8);
  if (!f || std::memcmp(magic, "\x93NUMPY", 6) != 0) throw std::runtime_error("Not a .npy file: " + path);
  size_t hlen = 0;
  if (magic[6] == 1) {
    unsigned char b[2];
    f.read(reinterpret_cast<char*>(b), 2);
    hlen = b[0] | (b[1] << 8);
  } else {
    unsigned char b[4];
    f.read(reinterpret_cast<char*>(b), 4);
    hlen = b[0] | (b[1] << 8) | (b[2] << 16) | (static_cast<size_t>(b[3]) << 24);
  }
  std::string header(hlen, ' ');
  f.read(&header[0], static_cast<std::streamsize>(hlen));
  if (header.find("'<f4'") == std::string::npos || header.find("'fortran_order': False") == std::string::npos ||
      header.find("(" + std::to_string(n) + ",)") == std::string::npos)
    throw std::runtime_error("Weights file " + path + " is not a float32 vector of " + std::to_string(n) + " values");
  std::vector<float> v(n);
  f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(float)));
  if (!f) throw std::runtime_error("Weights file " + path + " is truncated");
  return v;
}

std::string exe_dir(const char* argv0) {
  std::string p = argv0;
  const size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

lcr::PointCloud scaled(const lcr::PointCloud& in, float k) {
  lcr::PointCloud out = in;
  for (auto& p : out.points) {
    p.x *= k;
    p.y *= k;
    p.z *= k;
  }
  return out;
}

bool settled(const lcr_icp_result& r) { return r.converged && r.state != LCR_ICP_STATE_NO_CORRESPONDENCES && r.mse <= 16e-6; }

}  // namespace

int main(int argc, char* argv[]) {
  try {
    // Super4PCS takes both inputs after one -i: pull them out before option parsing
    std::vector<char*> rest{argv[0]};
    std::string P, Q;
    for (int a = 1; a < argc; ++a) {
      if ((!std::strcmp(argv[a], "-i") || !std::strcmp(argv[a], "--input")) && a + 1 < argc) {
        P = argv[++a];
        if (a + 1 < argc && argv[a + 1][0] != '-') Q = argv[++a];
      } else {
        rest.push_back(argv[a]);
      }
    }
    cli::Options desc("Options");
    desc.add("help,h", false, nullptr, "Print help message")
        .add("input,i", true, nullptr, "The two clouds: P (fixed) then Q (moved onto P)")
        .add("matrix,m", true, nullptr, "Output: the transform taking Q onto P (two header lines, then 4x4)")
        .add("registered,r", true, nullptr, "Output: Q transformed by that matrix (.ply)")
        .add("units,u", true, "1.0", "Metres per input unit")
        .add("refine", true, "1", "Refine the proposal with point-to-plane ICP (1) or not (0)")
        .add("weights,w", true, nullptr, "Network parameters (.npy, float32); default: the shipped ones")
        .add("time,t", true, nullptr, "Accepted for Super4PCS compatibility, ignored")
        .add("overlap,o", true, nullptr, "Accepted for Super4PCS compatibility, ignored")
        .add("delta,d", true, nullptr, "Accepted for Super4PCS compatibility, ignored")
        .add("samples,n", true, nullptr, "Accepted for Super4PCS compatibility, ignored");
    desc.parse(static_cast<int>(rest.size()), rest.data());
    if (desc.count("help")) {
      std::cout << "Learned coarse alignment of a pair of captures (pose network + ICP refinement)." << std::endl
                << std::endl;
      desc.print(std::cout);
      std::cout << std::endl;
      return 0;
    }
    if (P.empty() || Q.empty() || !desc.count("matrix"))
      throw std::logic_error("Correct mode of use: " + std::string(argv[0]) + " -i P.ply Q.ply -m matrix.txt");
    const double units = desc.num("units");
    if (!(units > 0)) throw std::logic_error("units must be positive");
    lcr::PointCloud::Ptr cp = cli::load_cloud(P), cq = cli::load_cloud(Q);
    if (!cp) throw std::runtime_error("Couldn't load input point cloud: " + P);
    if (!cq) throw std::runtime_error("Couldn't load input point cloud: " + Q);
    const std::string wpath =
        desc.count("weights") ? desc.str("weights") : exe_dir(argv[0]) + "/../weights/posenet.npy";
    const std::vector<float> params = load_npy_f32(wpath, LCR_POSENET_PARAMS);

    lcr::Context& ctx = lcr::Context::thread_default();
    lcr_posenet* net = nullptr;
    ctx.check(lcr_posenet_create(ctx.get(), 0, &net));
    std::shared_ptr<lcr_posenet> keep(net, [&ctx](lcr_posenet* n) { lcr_posenet_free(ctx.get(), n); });
    ctx.check(lcr_posenet_set_params(ctx.get(), net, params.data()));
    const float k = static_cast<float>(units);
    lcr::DeviceCloud dq(ctx, scaled(*cq, k)), dp(ctx, scaled(*cp, k));
    const lcr_cloud* src[1] = {dq.get()};
    const lcr_cloud* tgt[1] = {dp.get()};
    float T[16];
    ctx.check(lcr_posenet_propose(ctx.get(), net, src, tgt, 1, 0, T));
    if (std::atoi(desc.str("refine").c_str()) != 0) {
      lcr_icp_params p1, p2;
      lcr_icp_params_default(&p1);
      p1.method = LCR_ICP_POINT_TO_PLANE;
      p1.compute_fitness = 0;
      p1.transformation_epsilon = 1e-8;
      p1.euclidean_fitness_epsilon = 1e-7;
      p2 = p1;
      p1.max_correspondence_distance = 0.02;
      p1.max_iterations = 30;
      p2.max_correspondence_distance = 0.01;
      p2.max_iterations = 50;
      p2.transformation_epsilon = 1e-9;
      p2.euclidean_fitness_epsilon = 1e-8;
      auto refine = [&](const float* guess, lcr_icp_result& out) {
        lcr_icp_result r1;
        const lcr_status s1 = lcr_icp(ctx.get(), dq.get(), dp.get(), &p1, guess, &r1, nullptr);
        if (s1 != LCR_OK && s1 != LCR_ERR_NO_CORRESPONDENCES) ctx.check(s1);
        const lcr_status s2 = lcr_icp(ctx.get(), dq.get(), dp.get(), &p2, r1.transform, &out, nullptr);
        if (s2 != LCR_OK && s2 != LCR_ERR_NO_CORRESPONDENCES) ctx.check(s2);
        if (out.state == LCR_ICP_STATE_NO_CORRESPONDENCES) out = r1;
      };
      lcr_icp_result r;
      refine(T, r);
      if (!settled(r)) {  // plain ICP from centroid alignment
        float cpv[4], cqv[4];
        ctx.check(lcr_centroid(ctx.get(), dp.get(), cpv));
        ctx.check(lcr_centroid(ctx.get(), dq.get(), cqv));
        float G[16] = {1, 0, 0, cpv[0] - cqv[0], 0, 1, 0, cpv[1] - cqv[1], 0, 0, 1, cpv[2] - cqv[2], 0, 0, 0, 1};
        lcr_icp_result rf;
        refine(G, rf);
        if (settled(rf)) r = rf;
      }
      std::memcpy(T, r.transform, sizeof(T));
      std::cout << "Refined: " << (settled(r) ? "yes" : "no") << ", ICP iterations: " << r.iterations
                << ", inlier RMS (m): " << std::sqrt(r.mse) << std::endl;
    }
    // back to input units: the rotation is unit-free, the translation scales by 1/units
    lcr::Matrix4f M;
    for (int i = 0; i < 16; ++i) M.m[i] = T[i];
    for (int r = 0; r < 3; ++r) M(r, 3) = static_cast<float>(T[4 * r + 3] / units);
    std::ofstream mf(desc.str("matrix"));
    if (!mf) throw std::runtime_error("Unable to write matrix file: " + desc.str("matrix"));
    mf << "# pose_proposal: transform taking " << Q << " onto " << P << std::endl;
    mf << "# row-major 4x4, input units" << std::endl;
    mf << std::setprecision(9);
    for (int r = 0; r < 4; ++r)
      mf << M(r, 0) << " " << M(r, 1) << " " << M(r, 2) << " " << M(r, 3) << std::endl;
    if (desc.count("registered")) {
      lcr::PointCloud reg;
      lcr::transformPointCloudWithNormals(*cq, reg, M, ctx);
      cli::save_cloud(desc.str("registered"), reg);
    }
    cli::print_matrix(std::cout, M);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
  } catch (...) {
    std::cerr << "An unknown error has occurred." << std::endl;
  }
  return -1;
}
