// PCL-shaped C++ facade over liblcr (header-only; C++14).
//
// The classes mirror the PCL calls the reference tools make, with the same
// method names and argument meaning, so a PCL user's code ports by changing the
// namespace:
//   lcr::IterativeClosestPoint  -- pcl_tools/fine_registration.cpp:105-126
//   lcr::VoxelGrid              -- pcl_tools/cloud_downsampling.cpp:73-76
//   lcr::StatisticalOutlierRemoval -- pcl_tools/outlier_removal.cpp:80-84, :92
//   lcr::NormalEstimation       -- pcl_tools/normal_estimation.cpp:84-108
//   lcr::io::loadPLYFile / savePLYFileBinary, lcr::compute3DCentroid,
//   lcr::transformPointCloudWithNormals
// All compute runs on the GPU through the C ABI in lcr.h; errors throw
// lcr::Error carrying the lcr_status.
#ifndef LCR_PCL_HPP
#define LCR_PCL_HPP

#include <array>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lcr.h"

namespace lcr {

class Error : public std::runtime_error {
 public:
  Error(lcr_status s, const std::string& m) : std::runtime_error(m), status(s) {}
  lcr_status status;
};

typedef lcr_point PointXYZRGBNormal;

struct Matrix4f {
  std::array<float, 16> m;  // row-major
  float& operator()(int r, int c) { return m[4 * r + c]; }
  float operator()(int r, int c) const { return m[4 * r + c]; }
  static Matrix4f Identity() {
    Matrix4f I;
    I.m = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    return I;
  }
  bool isIdentity() const { return m == Identity().m; }
};

// Host cloud: PointCloud<PointXYZRGBNormal> with points in PCL's 48-byte layout.
class PointCloud {
 public:
  typedef std::shared_ptr<PointCloud> Ptr;
  std::vector<lcr_point> points;
  size_t size() const { return points.size(); }
  bool empty() const { return points.empty(); }
  PointCloud& operator+=(const PointCloud& o) {
    points.insert(points.end(), o.points.begin(), o.points.end());
    return *this;
  }
  PointCloud operator+(const PointCloud& o) const {
    PointCloud r(*this);
    r += o;
    return r;
  }
};

// One CUDA stream on one device; shared by the objects that use it.
class Context {
 public:
  Context() = default;  // empty handle; use Context(device) or thread_default()
  explicit Context(int device) {
    lcr_ctx* c = nullptr;
    const lcr_status s = lcr_ctx_create(&c, device);
    if (s != LCR_OK) throw Error(s, std::string("lcr_ctx_create: ") + lcr_status_string(s));
    h_ = std::shared_ptr<lcr_ctx>(c, lcr_ctx_destroy);
  }
  lcr_ctx* get() const { return h_.get(); }
  void check(lcr_status s) const {
    if (s != LCR_OK) throw Error(s, lcr_last_error(h_.get()));
  }
  // One context per host thread, created on first use.
  static Context& thread_default() {
    thread_local Context ctx(0);
    return ctx;
  }

 private:
  std::shared_ptr<lcr_ctx> h_;
};

// Device-resident cloud (RAII over lcr_cloud*).
class DeviceCloud {
 public:
  DeviceCloud() = default;
  DeviceCloud(const Context& ctx, const PointCloud& host) : ctx_(ctx) {
    lcr_cloud* c = nullptr;
    ctx.check(lcr_cloud_upload(ctx.get(), host.points.data(), host.points.size(), &c));
    reset(c);
  }
  DeviceCloud(const Context& ctx, lcr_cloud* c) : ctx_(ctx) { reset(c); }
  lcr_cloud* get() const { return c_.get(); }
  size_t size() const { return lcr_cloud_size(c_.get()); }
  void download(PointCloud& out) const {
    out.points.resize(size());
    ctx_.check(lcr_cloud_download(ctx_.get(), c_.get(), out.points.data(), out.points.size()));
  }

 private:
  void reset(lcr_cloud* c) {
    lcr_ctx* raw = ctx_.get();
    Context keep = ctx_;
    c_ = std::shared_ptr<lcr_cloud>(c, [raw, keep](lcr_cloud* p) { lcr_cloud_free(raw, p); });
  }
  Context ctx_;
  std::shared_ptr<lcr_cloud> c_;
};

namespace io {
inline int loadPLYFile(const std::string& path, PointCloud& cloud) {
  lcr_point* p = nullptr;
  size_t n = 0;
  if (lcr_ply_read(path.c_str(), &p, &n) != LCR_OK) return -1;
  cloud.points.assign(p, p + n);
  lcr_free(p);
  return 0;
}
inline int savePLYFileBinary(const std::string& path, const PointCloud& cloud) {
  return lcr_ply_write(path.c_str(), cloud.points.data(), cloud.points.size(), 1) == LCR_OK ? 0 : -1;
}
inline int savePLYFileASCII(const std::string& path, const PointCloud& cloud) {
  return lcr_ply_write(path.c_str(), cloud.points.data(), cloud.points.size(), 0) == LCR_OK ? 0 : -1;
}
}  // namespace io

class IterativeClosestPoint {
 public:
  explicit IterativeClosestPoint(const Context& ctx = Context::thread_default()) : ctx_(ctx) {
    lcr_icp_params_default(&p_);
  }
  void setInputSource(const PointCloud::Ptr& c) { src_ = DeviceCloud(ctx_, *c); }
  void setInputTarget(const PointCloud::Ptr& c) { tgt_ = DeviceCloud(ctx_, *c); }
  void setMaxCorrespondenceDistance(double d) { p_.max_correspondence_distance = d; }
  void setMaximumIterations(int n) { p_.max_iterations = n; }
  void setTransformationEpsilon(double e) { p_.transformation_epsilon = e; }
  void setEuclideanFitnessEpsilon(double e) { p_.euclidean_fitness_epsilon = e; }
  // Not in PCL's IterativeClosestPoint: selects the point-to-plane error
  // (PCL's TransformationEstimationPointToPlaneLLS); needs target normals.
  void setPointToPlane(bool on) { p_.method = on ? LCR_ICP_POINT_TO_PLANE : LCR_ICP_POINT_TO_POINT; }
  void align(PointCloud& output, const Matrix4f& guess = Matrix4f::Identity()) {
    lcr_cloud* reg = nullptr;
    const lcr_status s = lcr_icp(ctx_.get(), src_.get(), tgt_.get(), &p_, guess.m.data(), &res_, &reg);
    if (s != LCR_OK && s != LCR_ERR_NO_CORRESPONDENCES) ctx_.check(s);
    DeviceCloud(ctx_, reg).download(output);
  }
  Matrix4f getFinalTransformation() const {
    Matrix4f T;
    for (int i = 0; i < 16; ++i) T.m[i] = res_.transform[i];
    return T;
  }
  bool hasConverged() const { return res_.converged != 0; }
  double getFitnessScore() const { return res_.fitness; }
  const lcr_icp_result& result() const { return res_; }

 private:
  Context ctx_;
  lcr_icp_params p_;
  lcr_icp_result res_ = lcr_icp_result();
  DeviceCloud src_, tgt_;
};

class VoxelGrid {
 public:
  explicit VoxelGrid(const Context& ctx = Context::thread_default()) : ctx_(ctx) {}
  void setInputCloud(const PointCloud::Ptr& c) { in_ = DeviceCloud(ctx_, *c); }
  void setLeafSize(float lx, float ly, float lz) { l_ = {lx, ly, lz}; }
  void filter(PointCloud& out) {
    lcr_cloud* o = nullptr;
    ctx_.check(lcr_voxel_grid(ctx_.get(), in_.get(), l_[0], l_[1], l_[2], &o));
    DeviceCloud(ctx_, o).download(out);
  }

 private:
  Context ctx_;
  DeviceCloud in_;
  std::array<float, 3> l_ = {1.f, 1.f, 1.f};
};

class StatisticalOutlierRemoval {
 public:
  explicit StatisticalOutlierRemoval(const Context& ctx = Context::thread_default()) : ctx_(ctx) {}
  void setInputCloud(const PointCloud::Ptr& c) { in_ = DeviceCloud(ctx_, *c); }
  void setMeanK(int k) { k_ = k; }
  void setStddevMulThresh(double m) { mul_ = m; }
  void setNegative(bool n) { neg_ = n; }
  void filter(PointCloud& out) {
    lcr_cloud* o = nullptr;
    ctx_.check(lcr_sor(ctx_.get(), in_.get(), k_, mul_, neg_ ? nullptr : &o, neg_ ? &o : nullptr, &stats_));
    DeviceCloud(ctx_, o).download(out);
  }
  const lcr_sor_stats& stats() const { return stats_; }

 private:
  Context ctx_;
  DeviceCloud in_;
  int k_ = 1;
  double mul_ = 0.0;
  bool neg_ = false;
  lcr_sor_stats stats_ = lcr_sor_stats();
};

class NormalEstimation {
 public:
  explicit NormalEstimation(const Context& ctx = Context::thread_default()) : ctx_(ctx) {}
  void setInputCloud(const PointCloud::Ptr& c) { in_ = DeviceCloud(ctx_, *c); }
  void setKSearch(int k) { k_ = k; }
  void setViewPoint(float x, float y, float z) { vp_ = {x, y, z}; }
  // Clouds read from PLY carry the sensor origin (0, 0, 0).
  void useSensorOriginAsViewPoint() { vp_ = {0.f, 0.f, 0.f}; }
  // Output: the input cloud with normal_x/y/z and curvature filled in.
  void compute(PointCloud& out, bool flip_all = false) {
    lcr_cloud* o = nullptr;
    ctx_.check(lcr_normals(ctx_.get(), in_.get(), k_, vp_.data(), flip_all ? LCR_NORMALS_FLIP_ALL : 0, &o));
    DeviceCloud(ctx_, o).download(out);
  }

 private:
  Context ctx_;
  DeviceCloud in_;
  int k_ = 0;
  std::array<float, 3> vp_ = {0.f, 0.f, 0.f};
};

inline void compute3DCentroid(const PointCloud& cloud, std::array<float, 4>& c,
                              const Context& ctx = Context::thread_default()) {
  DeviceCloud d(ctx, cloud);
  ctx.check(lcr_centroid(ctx.get(), d.get(), c.data()));
}

inline void removeNaNFromPointCloud(const PointCloud& in, PointCloud& out,
                                   const Context& ctx = Context::thread_default()) {
  DeviceCloud d(ctx, in);
  lcr_cloud* o = nullptr;
  ctx.check(lcr_remove_nan(ctx.get(), d.get(), &o));
  DeviceCloud(ctx, o).download(out);
}

inline void transformPointCloudWithNormals(const PointCloud& in, PointCloud& out, const Matrix4f& T,
                                           const Context& ctx = Context::thread_default()) {
  DeviceCloud d(ctx, in);
  lcr_cloud* o = nullptr;
  ctx.check(lcr_transform(ctx.get(), d.get(), T.m.data(), &o));
  DeviceCloud(ctx, o).download(out);
}

}  // namespace lcr

#endif  // LCR_PCL_HPP
