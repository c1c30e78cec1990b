/*
 * CPU oracle for the alignment path -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Parity status: UNPINNED (the reference has no tests or golden data and its
 * PCL/FLANN/Eigen/OpenCV dependencies are absent).  Every function cites the
 * reference call site it restates.  Compile with -ffp-contract=off.
 */
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <queue>
#include <unordered_map>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const float kInf = std::numeric_limits<float>::infinity();

inline bool finite3(const orc_point& p) {
  return std::isfinite(p.x) && std::isfinite(p.y) && std::isfinite(p.z);
}

/* FLANN L2_Simple<float> on 3 components: result += diff*diff from 0, no FMA. */
inline float l2(float ax, float ay, float az, float bx, float by, float bz) {
  float d0 = ax - bx;
  float d1 = ay - by;
  float d2 = az - bz;
  float r = d0 * d0;
  r = r + d1 * d1;
  r = r + d2 * d2;
  return r;
}

/* ------------------------------------------------------------------------ */
/* Exact kd-tree.  Median split on the widest axis, leaves of <= 16 points.  */
/* Results ordered by (distance, index); ties resolved to the lower index.   */
/* ------------------------------------------------------------------------ */
struct KdTree {
  struct Node {
    int lo, hi;        // leaf range in order[]
    int axis;          // -1 for leaf
    float split;
    int left, right;
  };
  std::vector<float> x, y, z;  // reordered coordinates
  std::vector<int> id;         // original index of reordered slot
  std::vector<Node> nodes;

  void build(const orc_point* pts, size_t n) {
    std::vector<int> order;
    order.reserve(n);
    for (size_t i = 0; i < n; ++i)
      if (finite3(pts[i])) order.push_back(static_cast<int>(i));
    nodes.clear();
    nodes.reserve(2 * (order.size() / 8 + 1));
    if (!order.empty()) build_rec(pts, order, 0, static_cast<int>(order.size()));
    x.resize(order.size());
    y.resize(order.size());
    z.resize(order.size());
    id = order;
    for (size_t i = 0; i < order.size(); ++i) {
      x[i] = pts[order[i]].x;
      y[i] = pts[order[i]].y;
      z[i] = pts[order[i]].z;
    }
  }

  int build_rec(const orc_point* pts, std::vector<int>& order, int lo, int hi) {
    int me = static_cast<int>(nodes.size());
    nodes.push_back(Node{lo, hi, -1, 0.f, -1, -1});
    if (hi - lo <= 16) return me;
    float mn[3] = {kInf, kInf, kInf}, mx[3] = {-kInf, -kInf, -kInf};
    for (int i = lo; i < hi; ++i) {
      const orc_point& p = pts[order[i]];
      mn[0] = std::min(mn[0], p.x); mx[0] = std::max(mx[0], p.x);
      mn[1] = std::min(mn[1], p.y); mx[1] = std::max(mx[1], p.y);
      mn[2] = std::min(mn[2], p.z); mx[2] = std::max(mx[2], p.z);
    }
    int axis = 0;
    float ext = mx[0] - mn[0];
    if (mx[1] - mn[1] > ext) { axis = 1; ext = mx[1] - mn[1]; }
    if (mx[2] - mn[2] > ext) { axis = 2; }
    if (!(mx[axis] > mn[axis])) return me;  // all coincident: keep as a leaf
    int mid = (lo + hi) / 2;
    auto coord = [&](int i) { const orc_point& p = pts[i]; return axis == 0 ? p.x : (axis == 1 ? p.y : p.z); };
    std::nth_element(order.begin() + lo, order.begin() + mid, order.begin() + hi,
                     [&](int a, int b) { return coord(a) < coord(b); });
    float split = coord(order[mid]);
    nodes[me].axis = axis;
    nodes[me].split = split;
    int l = build_rec(pts, order, lo, mid);
    int r = build_rec(pts, order, mid, hi);
    nodes[me].left = l;
    nodes[me].right = r;
    return me;
  }

  typedef std::pair<float, int> Key;  // (distance, original index): lexicographic

  /* k nearest with every accepted distance <= cap.  Output sorted ascending. */
  void knn(float qx, float qy, float qz, int k, float cap, std::vector<Key>& out) const {
    std::priority_queue<Key> heap;  // max-heap on (dist, idx)
    if (!nodes.empty()) search(0, qx, qy, qz, k, cap, heap);
    out.resize(heap.size());
    for (int i = static_cast<int>(heap.size()) - 1; i >= 0; --i) {
      out[i] = heap.top();
      heap.pop();
    }
  }

  void search(int ni, float qx, float qy, float qz, int k, float cap, std::priority_queue<Key>& heap) const {
    const Node& nd = nodes[ni];
    if (nd.axis < 0) {
      for (int i = nd.lo; i < nd.hi; ++i) {
        float d = l2(qx, qy, qz, x[i], y[i], z[i]);
        if (!(d <= cap)) continue;
        Key c(d, id[i]);
        if (static_cast<int>(heap.size()) < k) heap.push(c);
        else if (c < heap.top()) { heap.pop(); heap.push(c); }
      }
      return;
    }
    float q = nd.axis == 0 ? qx : (nd.axis == 1 ? qy : qz);
    float diff = q - nd.split;
    int near_c = diff < 0 ? nd.left : nd.right;
    int far_c = diff < 0 ? nd.right : nd.left;
    search(near_c, qx, qy, qz, k, cap, heap);
    float bound = static_cast<int>(heap.size()) < k ? cap : heap.top().first;
    /* (q - split)^2 rounds below every far-side distance (monotone rounding), so
     * skipping on a strict '>' can never drop a point that ties the bound. */
    if (!(diff * diff > bound)) search(far_c, qx, qy, qz, k, cap, heap);
  }
};

/* Largest float f with (double)f <= v: the FP32 form of PCL's `dist > max_dist_sqr` test. */
float float_cap(double v) {
  if (!(v < static_cast<double>(FLT_MAX))) return kInf;
  float f = static_cast<float>(v);
  if (static_cast<double>(f) > v) f = std::nextafter(f, 0.0f);
  return f;
}

/* Fixed blocked summation order shared with the GPU reduction: blocks of 256
 * consecutive terms summed sequentially from 0.0, repeated until one value. */
/* The GPU's fixed order (the reference sums sequentially; the order only
 * moves the last bits of the SOR mean/stddev): chunks of 256 consecutive
 * terms; within a chunk, 32 partial sums p[l] of terms 8l..8l+7 in order from
 * 0.0, combined by the xor butterfly p[l] += p[l ^ o] for o = 16, 8, 4, 2, 1;
 * the chunk's sum is p[0].  Repeated until one value remains. */
double blocked_sum(std::vector<double> v) {
  if (v.empty()) return 0.0;
  while (v.size() > 1) {
    std::vector<double> next((v.size() + 255) / 256, 0.0);
    for (size_t b = 0; b < next.size(); ++b) {
      double p[32];
      for (int l = 0; l < 32; ++l) {
        double s = 0.0;
        for (int j = 0; j < 8; ++j) {
          const size_t i = b * 256 + static_cast<size_t>(l) * 8 + j;
          if (i < v.size()) s += v[i];
        }
        p[l] = s;
      }
      for (int o = 16; o > 0; o >>= 1) {
        double q[32];
        for (int l = 0; l < 32; ++l) q[l] = p[l] + p[l ^ o];
        for (int l = 0; l < 32; ++l) p[l] = q[l];
      }
      next[b] = p[0];
    }
    v.swap(next);
  }
  return v[0];
}

/* ---------------------------- small FP64 linear algebra ------------------ */

/* Symmetric 3x3 eigen-decomposition, cyclic Jacobi.  evals ascending, evecs columns. */
void eig3_jacobi(const double A[9], double w[3], double V[9]) {
  double a[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) a[i][j] = 0.5 * (A[3 * i + j] + A[3 * j + i]);
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    double diag = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off <= 1e-30 * diag || off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (a[p][q] == 0.0) continue;
        double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
  int ord[3] = {0, 1, 2};
  std::sort(ord, ord + 3, [&](int i, int j) { return a[i][i] < a[j][j]; });
  for (int c = 0; c < 3; ++c) {
    w[c] = a[ord[c]][ord[c]];
    for (int r = 0; r < 3; ++r) V[3 * r + c] = v[r][ord[c]];
  }
}

inline void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

double det3(const double M[9]) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
         M[2] * (M[3] * M[7] - M[4] * M[6]);
}

/* 3x3 SVD A = U diag(s) V^T through the eigen-decomposition of A^T A (oracle-only
 * route; the GPU uses one-sided Jacobi).  s descending. */
void svd3(const double A[9], double U[9], double s[3], double V[9]) {
  double AtA[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0;
      for (int k = 0; k < 3; ++k) acc += A[3 * k + i] * A[3 * k + j];
      AtA[3 * i + j] = acc;
    }
  double w[3], E[9];
  eig3_jacobi(AtA, w, E);  // ascending
  for (int c = 0; c < 3; ++c) {
    s[c] = std::sqrt(std::max(0.0, w[2 - c]));
    for (int r = 0; r < 3; ++r) V[3 * r + c] = E[3 * r + (2 - c)];
  }
  double u[3][3];
  for (int c = 0; c < 3; ++c) {
    for (int r = 0; r < 3; ++r) {
      double acc = 0;
      for (int k = 0; k < 3; ++k) acc += A[3 * r + k] * V[3 * k + c];
      u[c][r] = acc;
    }
  }
  double scale = s[0] > 0 ? s[0] : 1.0;
  for (int c = 0; c < 3; ++c) {
    double nrm = std::sqrt(u[c][0] * u[c][0] + u[c][1] * u[c][1] + u[c][2] * u[c][2]);
    bool ok = s[c] > 1e-12 * scale && nrm > 0;
    if (ok) {
      // Gram-Schmidt against previous columns for orthogonality
      for (int p = 0; p < c; ++p) {
        double d = u[c][0] * u[p][0] + u[c][1] * u[p][1] + u[c][2] * u[p][2];
        for (int r = 0; r < 3; ++r) u[c][r] -= d * u[p][r];
      }
      nrm = std::sqrt(u[c][0] * u[c][0] + u[c][1] * u[c][1] + u[c][2] * u[c][2]);
      ok = nrm > 1e-300;
    }
    if (ok) {
      for (int r = 0; r < 3; ++r) u[c][r] /= nrm;
    } else if (c == 2) {
      cross3(u[0], u[1], u[2]);
    } else {
      // pick an axis orthogonal to previous columns
      double cand[3] = {1, 0, 0};
      for (int tries = 0; tries < 3; ++tries) {
        cand[0] = tries == 0; cand[1] = tries == 1; cand[2] = tries == 2;
        for (int p = 0; p < c; ++p) {
          double d = cand[0] * u[p][0] + cand[1] * u[p][1] + cand[2] * u[p][2];
          for (int r = 0; r < 3; ++r) cand[r] -= d * u[p][r];
        }
        double cn = std::sqrt(cand[0] * cand[0] + cand[1] * cand[1] + cand[2] * cand[2]);
        if (cn > 0.5) { for (int r = 0; r < 3; ++r) u[c][r] = cand[r] / cn; break; }
      }
    }
  }
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) U[3 * r + c] = u[c][r];
}

/* Solve the SPD 6x6 system M x = b by LDL^T. Returns false if singular. */
/* SPD 6x6 solve by LDL^T; a pivot below 1e-12 of the largest diagonal entry
 * counts as singular (degenerate correspondence geometry). */
bool ldlt6(const double M[36], const double b[6], double x[6]) {
  double L[36] = {0}, D[6];
  double dmax = 0;
  for (int i = 0; i < 6; ++i) dmax = std::max(dmax, std::fabs(M[7 * i]));
  if (!(dmax > 0)) return false;
  for (int j = 0; j < 6; ++j) {
    double d = M[6 * j + j];
    for (int k = 0; k < j; ++k) d -= L[6 * j + k] * L[6 * j + k] * D[k];
    D[j] = d;
    if (!(d > 1e-12 * dmax)) return false;
    L[6 * j + j] = 1.0;
    for (int i = j + 1; i < 6; ++i) {
      double v = M[6 * i + j];
      for (int k = 0; k < j; ++k) v -= L[6 * i + k] * L[6 * j + k] * D[k];
      L[6 * i + j] = v / d;
    }
  }
  double y[6];
  for (int i = 0; i < 6; ++i) {
    double v = b[i];
    for (int k = 0; k < i; ++k) v -= L[6 * i + k] * y[k];
    y[i] = v;
  }
  for (int i = 0; i < 6; ++i) y[i] /= D[i];
  for (int i = 5; i >= 0; --i) {
    double v = y[i];
    for (int k = i + 1; k < 6; ++k) v -= L[6 * k + i] * x[k];
    x[i] = v;
  }
  return true;
}

/* Row-major 4x4 helpers. */
void mat4_mul(const double A[16], const double B[16], double C[16]) {
  double T[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += A[4 * i + k] * B[4 * k + j];
      T[4 * i + j] = s;
    }
  std::memcpy(C, T, sizeof(T));
}

/* Re-orthonormalise the rotation block (Gram-Schmidt on rows). */
void orthonormalize(double T[16]) {
  double r0[3] = {T[0], T[1], T[2]}, r1[3] = {T[4], T[5], T[6]}, r2[3];
  double n0 = std::sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
  for (int i = 0; i < 3; ++i) r0[i] /= n0;
  double d = r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2];
  for (int i = 0; i < 3; ++i) r1[i] -= d * r0[i];
  double n1 = std::sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  for (int i = 0; i < 3; ++i) r1[i] /= n1;
  cross3(r0, r1, r2);
  for (int i = 0; i < 3; ++i) { T[i] = r0[i]; T[4 + i] = r1[i]; T[8 + i] = r2[i]; }
}

/* The FP32 rigid transform used for every correspondence pass: float cast of the
 * FP64 state, applied as ((r0*x + r1*y) + r2*z) + t (Eigen's evaluation order). */
struct Xf32 {
  float m[12];
  explicit Xf32(const double* T) { for (int i = 0; i < 12; ++i) m[i] = static_cast<float>(T[i]); }
  inline void apply(float x, float y, float z, float& ox, float& oy, float& oz) const {
    float a, b;
    a = m[0] * x; b = m[1] * y; a = a + b; b = m[2] * z; a = a + b; ox = a + m[3];
    a = m[4] * x; b = m[5] * y; a = a + b; b = m[6] * z; a = a + b; oy = a + m[7];
    a = m[8] * x; b = m[9] * y; a = a + b; b = m[10] * z; a = a + b; oz = a + m[11];
  }
};

int g_threads = 0;
inline int nthreads() {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

void orc_set_threads(int n) { g_threads = n; }

/* super_resolution.cpp:295-309 and :315.  The per-pixel mean of the non-zero
 * samples is taken in double (mean() :19-23) and returned as float; the image
 * is then converted to CV_16UC1 (round to nearest even, saturate).  With no
 * non-zero sample the reference divides 0.0 by 0 (NaN), which the conversion
 * saturates to 0. */
void orc_ze_mean_u16(const uint16_t* frames, int nframes, size_t npix, uint16_t* out) {
  for (size_t p = 0; p < npix; ++p) {
    double sum = 0.0;
    size_t cnt = 0;
    for (int f = 0; f < nframes; ++f) {
      float v = static_cast<float>(frames[static_cast<size_t>(f) * npix + p]);
      if (v > 0) { sum += v; ++cnt; }
    }
    if (cnt == 0) { out[p] = 0; continue; }
    float m = static_cast<float>(sum / static_cast<double>(cnt));
    float r = std::nearbyint(m);  // default rounding mode: nearest even
    out[p] = r <= 0 ? 0 : (r >= 65535.f ? 65535 : static_cast<uint16_t>(r));
  }
}

/* super_resolution_kv2.cpp:287-303: same mean, guarded when no sample exists
 * (the pixel then keeps its initial value; 0 here). */
void orc_ze_mean_f32(const float* frames, int nframes, size_t npix, float* out) {
  for (size_t p = 0; p < npix; ++p) {
    double sum = 0.0;
    size_t cnt = 0;
    for (int f = 0; f < nframes; ++f) {
      float v = frames[static_cast<size_t>(f) * npix + p];
      if (v > 0) { sum += v; ++cnt; }
    }
    out[p] = cnt ? static_cast<float>(sum / static_cast<double>(cnt)) : 0.0f;
  }
}

/* depth_capture.cpp:231-265: central differences with rows as the x direction
 * (i+-1) and columns as y (j+-1), 20 mm discontinuity threshold, zero
 * neighbours on the image border, d = (-dzdx, -dzdy, 1) normalised as
 * cv::normalize does (multiply by 1/||d||), stored as float. */
void orc_image_normals_u16(const uint16_t* depth, int w, int h, float* nrm) {
  for (int i = 0; i < h; ++i)
    for (int j = 0; j < w; ++j) {
      int c = depth[static_cast<size_t>(i) * w + j];
      int right = 0, left = 0, down = 0, up = 0;
      if (i > 0 && j > 0 && i < h - 1 && j < w - 1) {
        right = depth[static_cast<size_t>(i + 1) * w + j];
        left = depth[static_cast<size_t>(i - 1) * w + j];
        down = depth[static_cast<size_t>(i) * w + j + 1];
        up = depth[static_cast<size_t>(i) * w + j - 1];
      }
      if (std::abs(c - right) > 20) right = 0;
      if (std::abs(c - left) > 20) left = 0;
      if (std::abs(c - down) > 20) down = 0;
      if (std::abs(c - up) > 20) up = 0;
      double dzdx = (right - left) / 2.0;
      double dzdy = (down - up) / 2.0;
      double d0 = -dzdx, d1 = -dzdy, d2 = 1.0;
      double s = d0 * d0;
      s = s + d1 * d1;
      s = s + d2 * d2;
      double nv = std::sqrt(s);
      double inv = nv != 0.0 ? 1.0 / nv : 0.0;
      float* o = nrm + 3 * (static_cast<size_t>(i) * w + j);
      o[0] = static_cast<float>(d0 * inv);
      o[1] = static_cast<float>(d1 * inv);
      o[2] = static_cast<float>(d2 * inv);
    }
}

/* depth_capture.cpp:267-308 (same arithmetic as super_resolution.cpp:79-117):
 * pixels kept when z != 0, depth_min <= z <= depth_max and inside the ROI;
 * x = z*(j-cx)*(1/fx), y = -z*(i-cy)*(1/fy), z' = -z, evaluated in double.
 * Output in row-major pixel order, multiplied by `scale` in double and rounded
 * once to float.  ascii_roundtrip=1 instead reproduces the reference's
 * fprintf("%.6lf") + PCL text parse (only meaningful with scale == 1). */
size_t orc_backproject_v1(const uint16_t* depth, const orc_bp_params* p, int ascii_roundtrip, orc_point* out) {
  const int w = p->width, h = p->height;
  std::vector<float> nrm;
  if (p->normals) {
    nrm.resize(static_cast<size_t>(w) * h * 3);
    orc_image_normals_u16(depth, w, h, nrm.data());
  }
  const double ifx = 1 / p->fx, ify = 1 / p->fy;
  size_t n = 0;
  char buf[64];
  for (int i = 0; i < h; ++i)
    for (int j = 0; j < w; ++j) {
      uint16_t z = depth[static_cast<size_t>(i) * w + j];
      if (!(z != 0 && z >= p->depth_min && z <= p->depth_max && i >= p->roi_top && i <= p->roi_bottom &&
            j >= p->roi_left && j <= p->roi_right))
        continue;
      double vx = static_cast<double>(z) * (j - p->cx) * ifx;
      double vy = static_cast<double>(-static_cast<int>(z)) * (i - p->cy) * ify;
      double vz = static_cast<double>(-static_cast<int>(z));
      orc_point& o = out[n++];
      std::memset(&o, 0, sizeof(o));
      if (ascii_roundtrip) {
        std::snprintf(buf, sizeof buf, "%.6lf", vx); o.x = std::strtof(buf, nullptr);
        std::snprintf(buf, sizeof buf, "%.6lf", vy); o.y = std::strtof(buf, nullptr);
        std::snprintf(buf, sizeof buf, "%.6lf", vz); o.z = std::strtof(buf, nullptr);
      } else {
        o.x = static_cast<float>(vx * p->scale);
        o.y = static_cast<float>(vy * p->scale);
        o.z = static_cast<float>(vz * p->scale);
      }
      if (p->normals) {
        const float* nn = &nrm[3 * (static_cast<size_t>(i) * w + j)];
        o.normal_x = nn[0]; o.normal_y = nn[1]; o.normal_z = nn[2];
      }
      o.r = p->r; o.g = p->g; o.b = p->b;
    }
  return n;
}

/* kinect2.h:256-267 (colmap/rowmap), :169-187 (per-pixel depth/1000, NaN and
 * |d|<1e-4 rejection, x = colmap*d, y = -rowmap*d, z = -d), then
 * depth_capture_kv2.cpp:233-256: reprojection ROI test and the uniform scale
 * (an Affine3f, i.e. one float multiply per coordinate).  Camera parameters are
 * floats as in libfreenect2's IrCameraParams. */
size_t orc_backproject_v2(const float* depth_mm, const orc_bp_params* p, orc_point* out) {
  const int w = p->width, h = p->height;
  const float fx = static_cast<float>(p->fx), fy = static_cast<float>(p->fy);
  const float cx = static_cast<float>(p->cx), cy = static_cast<float>(p->cy);
  const float sc = static_cast<float>(p->scale);
  std::vector<float> colmap(w), rowmap(h);
  for (int i = 0; i < w; ++i) colmap[i] = static_cast<float>((i - cx + 0.5) / fx);
  for (int i = 0; i < h; ++i) rowmap[i] = static_cast<float>((i - cy + 0.5) / fy);
  size_t n = 0;
  for (int yy = 0; yy < h; ++yy)
    for (int xx = 0; xx < w; ++xx) {
      const float dv = depth_mm[static_cast<size_t>(yy) * w + xx] / 1000.0f;
      if (std::isnan(dv) || std::fabs(dv) < 0.0001) continue;
      const float rx = colmap[xx] * dv;
      const float ry = rowmap[yy] * dv;
      const float px = rx, py = -ry, pz = -dv;
      const float X = static_cast<float>(((px / (-pz)) * fx) - 0.5 + cx);
      const float Y = static_cast<float>((((-py) / (-pz)) * fy) - 0.5 + cy);
      const float D = static_cast<float>((-pz) * 1000.0);
      if (!(D != 0 && D >= p->depth_min && D <= p->depth_max && Y >= p->roi_top && Y <= p->roi_bottom &&
            X >= p->roi_left && X <= p->roi_right))
        continue;
      orc_point& o = out[n++];
      std::memset(&o, 0, sizeof(o));
      o.x = sc * px; o.y = sc * py; o.z = sc * pz;
      o.r = p->r; o.g = p->g; o.b = p->b;
    }
  return n;
}

int orc_knn(const orc_point* ref, size_t m, const orc_point* q, size_t n, int k, float max_dist_sq,
            int32_t* idx, float* dist) {
  if (k <= 0) return -1;
  KdTree tree;
  tree.build(ref, m);
  const float cap = max_dist_sq < 0 ? kInf : max_dist_sq;
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(n); ++i) {
    std::vector<KdTree::Key> res;
    if (finite3(q[i])) tree.knn(q[i].x, q[i].y, q[i].z, k, cap, res);
    for (int j = 0; j < k; ++j) {
      if (j < static_cast<int>(res.size())) {
        idx[i * k + j] = res[j].second;
        dist[i * k + j] = res[j].first;
      } else {
        idx[i * k + j] = -1;
        dist[i * k + j] = kInf;
      }
    }
  }
  return 0;
}

/* ----------------------------------------------------------------------- */
/* VoxelGrid (cloud_downsampling.cpp:73-76)                                 */
/* ----------------------------------------------------------------------- */
namespace {
struct VoxelSetup {
  bool overflow = false;
  bool empty = true;
  float inv[3];
  int min_b[3], div_b[3];
};

VoxelSetup voxel_setup(const orc_point* in, size_t n, float lx, float ly, float lz) {
  VoxelSetup s;
  const float leaf[3] = {lx, ly, lz};
  for (int a = 0; a < 3; ++a) s.inv[a] = 1.0f / leaf[a];
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (size_t i = 0; i < n; ++i) {
    if (!finite3(in[i])) continue;
    s.empty = false;
    const float c[3] = {in[i].x, in[i].y, in[i].z};
    for (int a = 0; a < 3; ++a) { mn[a] = std::min(mn[a], c[a]); mx[a] = std::max(mx[a], c[a]); }
  }
  if (s.empty) return s;
  int64_t d[3];
  for (int a = 0; a < 3; ++a) {
    float ext = mx[a] - mn[a];
    float cells = ext * s.inv[a];
    if (!(cells < 9.0e18f)) {  // would not fit int64: PCL's product overflows (undefined); refuse
      s.overflow = true;
      return s;
    }
    d[a] = static_cast<int64_t>(cells) + 1;
  }
  // PCL tests dx*dy*dz > INT32_MAX in int64, which itself overflows for huge
  // ranges; the product is checked in double first so those refuse as well.
  const double prod = static_cast<double>(d[0]) * static_cast<double>(d[1]) * static_cast<double>(d[2]);
  if (prod > 2147483647.0 || d[0] * d[1] * d[2] > static_cast<int64_t>(std::numeric_limits<int32_t>::max())) {
    s.overflow = true;
    return s;
  }
  for (int a = 0; a < 3; ++a) {
    float lo = mn[a] * s.inv[a], hi = mx[a] * s.inv[a];
    s.min_b[a] = static_cast<int>(std::floor(lo));
    int max_b = static_cast<int>(std::floor(hi));
    s.div_b[a] = max_b - s.min_b[a] + 1;
  }
  return s;
}

inline int64_t voxel_key(const VoxelSetup& s, const orc_point& p) {
  const float c[3] = {p.x, p.y, p.z};
  int ijk[3];
  for (int a = 0; a < 3; ++a) {
    float v = c[a] * s.inv[a];
    ijk[a] = static_cast<int>(std::floor(v) - static_cast<float>(s.min_b[a]));
  }
  int idx = ijk[0] + ijk[1] * s.div_b[0] + ijk[2] * (s.div_b[0] * s.div_b[1]);
  return static_cast<int64_t>(static_cast<uint32_t>(idx));
}
}  // namespace

void orc_voxel_keys(const orc_point* in, size_t n, float lx, float ly, float lz, int64_t* keys) {
  VoxelSetup s = voxel_setup(in, n, lx, ly, lz);
  for (size_t i = 0; i < n; ++i) keys[i] = (s.empty || s.overflow || !finite3(in[i])) ? -1 : voxel_key(s, in[i]);
}

/* Points are grouped by voxel index (ascending); within a voxel they are summed
 * in ascending input order (the stated order: PCL sorts with the unstable
 * std::sort, so its within-voxel order is unspecified).  Every field is
 * averaged in float and divided by float(count); r, g, b are averaged as
 * floats and truncated, alpha becomes 0 (PCL packs (r<<16)|(g<<8)|b). */
size_t orc_voxel_grid(const orc_point* in, size_t n, float lx, float ly, float lz, orc_point* out, int* overflow) {
  VoxelSetup s = voxel_setup(in, n, lx, ly, lz);
  if (overflow) *overflow = s.overflow ? 1 : 0;
  if (s.empty) return 0;
  if (s.overflow) {
    std::memcpy(out, in, n * sizeof(orc_point));
    return n;
  }
  std::vector<std::pair<uint32_t, uint32_t>> iv;
  iv.reserve(n);
  for (size_t i = 0; i < n; ++i)
    if (finite3(in[i])) iv.emplace_back(static_cast<uint32_t>(voxel_key(s, in[i])), static_cast<uint32_t>(i));
  std::stable_sort(iv.begin(), iv.end(),
                   [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                     return a.first < b.first;
                   });
  size_t no = 0;
  for (size_t f = 0; f < iv.size();) {
    size_t l = f + 1;
    while (l < iv.size() && iv[l].first == iv[f].first) ++l;
    float acc[10];
    const orc_point& p0 = in[iv[f].second];
    acc[0] = p0.x; acc[1] = p0.y; acc[2] = p0.z;
    acc[3] = p0.normal_x; acc[4] = p0.normal_y; acc[5] = p0.normal_z; acc[6] = p0.curvature;
    acc[7] = p0.r; acc[8] = p0.g; acc[9] = p0.b;
    for (size_t i = f + 1; i < l; ++i) {
      const orc_point& p = in[iv[i].second];
      acc[0] += p.x; acc[1] += p.y; acc[2] += p.z;
      acc[3] += p.normal_x; acc[4] += p.normal_y; acc[5] += p.normal_z; acc[6] += p.curvature;
      acc[7] += static_cast<float>(p.r); acc[8] += static_cast<float>(p.g); acc[9] += static_cast<float>(p.b);
    }
    const float cnt = static_cast<float>(l - f);
    orc_point& o = out[no++];
    std::memset(&o, 0, sizeof(o));
    o.x = acc[0] / cnt; o.y = acc[1] / cnt; o.z = acc[2] / cnt;
    o.normal_x = acc[3] / cnt; o.normal_y = acc[4] / cnt; o.normal_z = acc[5] / cnt;
    o.curvature = acc[6] / cnt;
    o.r = static_cast<uint8_t>(static_cast<int>(acc[7] / cnt));
    o.g = static_cast<uint8_t>(static_cast<int>(acc[8] / cnt));
    o.b = static_cast<uint8_t>(static_cast<int>(acc[9] / cnt));
    o.a = 0;
    f = l;
  }
  return no;
}

/* ----------------------------------------------------------------------- */
/* StatisticalOutlierRemoval (outlier_removal.cpp:80-84, accumulate :114-118) */
/* ----------------------------------------------------------------------- */
int orc_sor(const orc_point* in, size_t n, int mean_k, double std_mul, int sqrt_double, int sum_mode,
            float* distances, uint8_t* keep, double* stats) {
  if (mean_k <= 0) return -1;
  size_t nfinite = 0;
  for (size_t i = 0; i < n; ++i) nfinite += finite3(in[i]);
  if (static_cast<size_t>(mean_k) + 1 > nfinite) return -2;  // PCL would read past its k+1 results
  KdTree tree;
  tree.build(in, n);
  std::vector<char> valid(n, 0);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(n); ++i) {
    if (!finite3(in[i])) { distances[i] = 0.0f; continue; }
    std::vector<KdTree::Key> res;
    tree.knn(in[i].x, in[i].y, in[i].z, mean_k + 1, kInf, res);
    double dist_sum = 0.0;
    for (int k = 1; k < mean_k + 1; ++k) {
      if (sqrt_double) dist_sum += std::sqrt(static_cast<double>(res[k].first));
      else dist_sum += std::sqrt(res[k].first);
    }
    distances[i] = static_cast<float>(dist_sum / mean_k);
    valid[i] = 1;
  }
  size_t nvalid = 0;
  for (size_t i = 0; i < n; ++i) nvalid += valid[i];
  double sum = 0, sq_sum = 0;
  if (sum_mode == 1) {
    for (size_t i = 0; i < n; ++i) {
      sum += distances[i];
      sq_sum += distances[i] * distances[i];
    }
  } else {
    std::vector<double> a(n), b(n);
    for (size_t i = 0; i < n; ++i) { a[i] = distances[i]; b[i] = distances[i] * distances[i]; }
    sum = blocked_sum(a);
    sq_sum = blocked_sum(b);
  }
  const double nv = static_cast<double>(nvalid);
  double mean = sum / nv;
  double variance = (sq_sum - sum * sum / nv) / (nv - 1);
  double stddev = std::sqrt(variance);
  double thr = mean + std_mul * stddev;
  for (size_t i = 0; i < n; ++i) keep[i] = distances[i] > thr ? 0 : 1;
  if (stats) { stats[0] = mean; stats[1] = stddev; stats[2] = thr; stats[3] = nv; }
  return 0;
}

/* ----------------------------------------------------------------------- */
/* NormalEstimation (normal_estimation.cpp:84-118), FP64                    */
/* ----------------------------------------------------------------------- */
int orc_normals(const orc_point* in, size_t n, int k, const float* vp, int flip_all, orc_point* out) {
  if (k <= 0) return -1;
  KdTree tree;
  tree.build(in, n);
  const float nan = std::numeric_limits<float>::quiet_NaN();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(n); ++i) {
    orc_point o = in[i];
    std::vector<KdTree::Key> res;
    if (finite3(in[i])) tree.knn(in[i].x, in[i].y, in[i].z, k, kInf, res);
    if (res.size() < 3) {
      o.normal_x = o.normal_y = o.normal_z = o.curvature = nan;
      out[i] = o;
      continue;
    }
    double mu[3] = {0, 0, 0};
    for (auto& r : res) { mu[0] += in[r.second].x; mu[1] += in[r.second].y; mu[2] += in[r.second].z; }
    const double cnt = static_cast<double>(res.size());
    for (int a = 0; a < 3; ++a) mu[a] /= cnt;
    double C[9] = {0};
    for (auto& r : res) {
      double d[3] = {in[r.second].x - mu[0], in[r.second].y - mu[1], in[r.second].z - mu[2]};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) C[3 * a + b] += d[a] * d[b];
    }
    for (int a = 0; a < 9; ++a) C[a] /= cnt;
    bool zero = true;
    for (int a = 0; a < 9; ++a) zero = zero && C[a] == 0.0;
    if (zero) {  // all neighbours coincide: NaN normal, curvature 0 (as PCL's eigen33 + solvePlaneParameters)
      o.normal_x = o.normal_y = o.normal_z = nan;
      o.curvature = 0.f;
      out[i] = o;
      continue;
    }
    double w[3], V[9];
    eig3_jacobi(C, w, V);
    double nx = V[0], ny = V[3], nz = V[6];
    double tr = C[0] + C[4] + C[8];
    double curv = tr != 0 ? std::fabs(w[0] / tr) : 0.0;
    double cs = (vp[0] - in[i].x) * nx + (vp[1] - in[i].y) * ny + (vp[2] - in[i].z) * nz;
    if (cs < 0) { nx = -nx; ny = -ny; nz = -nz; }
    if (flip_all) { nx = -nx; ny = -ny; nz = -nz; }
    o.normal_x = static_cast<float>(nx);
    o.normal_y = static_cast<float>(ny);
    o.normal_z = static_cast<float>(nz);
    o.curvature = static_cast<float>(curv);
    out[i] = o;
  }
  return 0;
}

/* ----------------------------------------------------------------------- */
/* IterativeClosestPoint (fine_registration.cpp:105-126)                     */
/* ----------------------------------------------------------------------- */
namespace {

struct Corr {
  int s, t;
  float d;
};

void find_corr(const KdTree& tree, const orc_point* src, size_t ns, const double* T, float cap,
               std::vector<Corr>& out, std::vector<float>& tx) {
  Xf32 xf(T);
  std::vector<int> best(ns, -1);
  std::vector<float> bd(ns, kInf);
  tx.resize(3 * ns);
#pragma omp parallel for schedule(dynamic, 512) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(ns); ++i) {
    float x, y, z;
    xf.apply(src[i].x, src[i].y, src[i].z, x, y, z);
    tx[3 * i] = x; tx[3 * i + 1] = y; tx[3 * i + 2] = z;
    if (!finite3(src[i])) continue;
    std::vector<KdTree::Key> res;
    tree.knn(x, y, z, 1, cap, res);
    if (!res.empty()) { best[i] = res[0].second; bd[i] = res[0].first; }
  }
  out.clear();
  for (size_t i = 0; i < ns; ++i)
    if (best[i] >= 0) out.push_back(Corr{static_cast<int>(i), best[i], bd[i]});
}

/* Point-to-point: Umeyama without scale (PCL's default TransformationEstimationSVD),
 * two-pass FP64. */
void estimate_p2p(const std::vector<Corr>& corr, const std::vector<float>& tx, const orc_point* tgt, double dT[16]) {
  const double n = static_cast<double>(corr.size());
  double ms[3] = {0, 0, 0}, mt[3] = {0, 0, 0};
  for (const Corr& c : corr) {
    for (int a = 0; a < 3; ++a) ms[a] += tx[3 * c.s + a];
    mt[0] += tgt[c.t].x; mt[1] += tgt[c.t].y; mt[2] += tgt[c.t].z;
  }
  for (int a = 0; a < 3; ++a) { ms[a] /= n; mt[a] /= n; }
  double S[9] = {0};
  for (const Corr& c : corr) {
    double ds[3] = {tx[3 * c.s] - ms[0], tx[3 * c.s + 1] - ms[1], tx[3 * c.s + 2] - ms[2]};
    double dt[3] = {tgt[c.t].x - mt[0], tgt[c.t].y - mt[1], tgt[c.t].z - mt[2]};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) S[3 * a + b] += dt[a] * ds[b];
  }
  for (int a = 0; a < 9; ++a) S[a] /= n;
  double U[9], sv[3], V[9];
  svd3(S, U, sv, V);
  double D = (det3(U) * det3(V) < 0) ? -1.0 : 1.0;
  double R[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = U[3 * i + 0] * V[3 * j + 0] + U[3 * i + 1] * V[3 * j + 1] + D * U[3 * i + 2] * V[3 * j + 2];
  std::memset(dT, 0, 16 * sizeof(double));
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) dT[4 * i + j] = R[3 * i + j];
    dT[4 * i + 3] = mt[i] - (R[3 * i] * ms[0] + R[3 * i + 1] * ms[1] + R[3 * i + 2] * ms[2]);
  }
  dT[15] = 1.0;
}

/* R = Rz(gamma) Ry(beta) Rx(alpha): the Euler convention of PCL's point-to-plane
 * linear least squares (constructTransformationMatrix). */
void euler_zyx(double al, double be, double ga, double R[9]) {
  double ca = std::cos(al), sa = std::sin(al), cb = std::cos(be), sb = std::sin(be), cg = std::cos(ga), sg = std::sin(ga);
  R[0] = cg * cb; R[1] = -sg * ca + cg * sb * sa; R[2] = sg * sa + cg * sb * ca;
  R[3] = sg * cb; R[4] = cg * ca + sg * sb * sa;  R[5] = -cg * sa + sg * sb * ca;
  R[6] = -sb;     R[7] = cb * sa;                 R[8] = cb * ca;
}

/* Point-to-plane linearised least squares about the fixed centre c (the target
 * centroid): rows [ (s-c) x n , n ], rhs n.(d - s).  FP64 normal equations,
 * LDL^T solve. */
bool estimate_p2pl(const std::vector<Corr>& corr, const std::vector<float>& tx, const orc_point* tgt,
                   const double c[3], double dT[16]) {
  double M[36] = {0}, b[6] = {0};
  for (const Corr& cr : corr) {
    double s[3] = {tx[3 * cr.s] - c[0], tx[3 * cr.s + 1] - c[1], tx[3 * cr.s + 2] - c[2]};
    double d[3] = {tgt[cr.t].x - c[0], tgt[cr.t].y - c[1], tgt[cr.t].z - c[2]};
    double nn[3] = {tgt[cr.t].normal_x, tgt[cr.t].normal_y, tgt[cr.t].normal_z};
    if (!(std::isfinite(nn[0]) && std::isfinite(nn[1]) && std::isfinite(nn[2]))) continue;
    double a[6];
    cross3(s, nn, a);
    a[3] = nn[0]; a[4] = nn[1]; a[5] = nn[2];
    double r = nn[0] * (d[0] - s[0]) + nn[1] * (d[1] - s[1]) + nn[2] * (d[2] - s[2]);
    for (int i = 0; i < 6; ++i) {
      for (int j = 0; j < 6; ++j) M[6 * i + j] += a[i] * a[j];
      b[i] += a[i] * r;
    }
  }
  double x[6];
  if (!ldlt6(M, b, x)) return false;
  double R[9];
  euler_zyx(x[0], x[1], x[2], R);
  std::memset(dT, 0, 16 * sizeof(double));
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) dT[4 * i + j] = R[3 * i + j];
    dT[4 * i + 3] = x[3 + i] + c[i] - (R[3 * i] * c[0] + R[3 * i + 1] * c[1] + R[3 * i + 2] * c[2]);
  }
  dT[15] = 1.0;
  return true;
}

}  // namespace

int orc_correspondences(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt, const double* T,
                        double max_corr_dist, int32_t* idx, float* dist) {
  KdTree tree;
  tree.build(tgt, nt);
  float cap = float_cap(max_corr_dist * max_corr_dist);
  Xf32 xf(T);
#pragma omp parallel for schedule(dynamic, 512) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(ns); ++i) {
    idx[i] = -1; dist[i] = kInf;
    if (!finite3(src[i])) continue;
    float x, y, z;
    xf.apply(src[i].x, src[i].y, src[i].z, x, y, z);
    std::vector<KdTree::Key> res;
    tree.knn(x, y, z, 1, cap, res);
    if (!res.empty()) { idx[i] = res[0].second; dist[i] = res[0].first; }
  }
  return 0;
}

double orc_fitness(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt, const double* T) {
  KdTree tree;
  tree.build(tgt, nt);
  Xf32 xf(T);
  std::vector<float> d(ns, -1.0f);
#pragma omp parallel for schedule(dynamic, 512) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(ns); ++i) {
    if (!finite3(src[i])) continue;
    float x, y, z;
    xf.apply(src[i].x, src[i].y, src[i].z, x, y, z);
    std::vector<KdTree::Key> res;
    tree.knn(x, y, z, 1, kInf, res);
    if (!res.empty()) d[i] = res[0].first;
  }
  double s = 0;
  long long nr = 0;
  for (size_t i = 0; i < ns; ++i)
    if (d[i] >= 0) { s += d[i]; ++nr; }
  return nr > 0 ? s / nr : DBL_MAX;
}

/* The loop of pcl::IterativeClosestPoint::computeTransformation with
 * DefaultConvergenceCriteria as configured by the reference tool
 * (fine_registration.cpp:112-118): translation threshold = epsilon, rotation
 * threshold = 1 - epsilon, relative MSE = euclidean_fitness_epsilon, absolute
 * MSE 1e-12, no similar-iteration grace, and reaching max_iterations counts as
 * converged.  The increment is judged on its float cast, as PCL's Matrix4f. */
int orc_icp(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt, const orc_icp_params* prm,
            const double* guess, orc_icp_result* res) {
  std::memset(res, 0, sizeof(*res));
  double T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  if (guess) std::memcpy(T, guess, sizeof(T));
  std::memcpy(res->transform, T, sizeof(T));
  if (ns == 0 || nt == 0) { res->fitness = DBL_MAX; return -1; }
  KdTree tree;
  tree.build(tgt, nt);
  double c[3] = {0, 0, 0};
  {
    size_t cnt = 0;
    for (size_t i = 0; i < nt; ++i)
      if (finite3(tgt[i])) { c[0] += tgt[i].x; c[1] += tgt[i].y; c[2] += tgt[i].z; ++cnt; }
    for (int a = 0; a < 3; ++a) c[a] = static_cast<float>(c[a] / (cnt ? cnt : 1));
  }
  const float cap = float_cap(prm->max_corr_dist * prm->max_corr_dist);
  const int min_corr = prm->min_correspondences > 0 ? prm->min_correspondences : 3;
  double prev_mse = DBL_MAX;
  int iters = 0;
  std::vector<Corr> corr;
  std::vector<float> tx;
  int converged = 0, state = 0;
  for (;;) {
    find_corr(tree, src, ns, T, cap, corr, tx);
    res->n_corr_last = static_cast<int>(corr.size());
    if (static_cast<int>(corr.size()) < min_corr) { converged = 0; state = 5; break; }
    double dT[16];
    if (prm->point_to_plane) {
      if (!estimate_p2pl(corr, tx, tgt, c, dT)) { converged = 0; state = 5; break; }
    } else {
      estimate_p2p(corr, tx, tgt, dT);
    }
    mat4_mul(dT, T, T);
    orthonormalize(T);
    ++iters;
    double mse = 0;
    for (const Corr& cr : corr) mse += cr.d;
    mse /= static_cast<double>(corr.size());
    res->mse_last = mse;
    if (iters >= prm->max_iterations) { converged = 1; state = 1; break; }
    float f[16];
    for (int i = 0; i < 16; ++i) f[i] = static_cast<float>(dT[i]);
    double cos_angle = 0.5 * (static_cast<double>(f[0]) + f[5] + f[10] - 1);
    double tsq = static_cast<double>(f[3]) * f[3] + static_cast<double>(f[7]) * f[7] + static_cast<double>(f[11]) * f[11];
    if (cos_angle >= 1.0 - prm->transformation_epsilon && tsq <= prm->transformation_epsilon) {
      converged = 1; state = 2; break;
    }
    if (std::fabs(mse - prev_mse) < 1e-12) { converged = 1; state = 3; break; }
    if (std::fabs(mse - prev_mse) / prev_mse < prm->euclidean_fitness_epsilon) { converged = 1; state = 4; break; }
    prev_mse = mse;
  }
  std::memcpy(res->transform, T, sizeof(T));
  res->converged = converged;
  res->iterations = iters;
  res->state = state;
  res->fitness = orc_fitness(src, ns, tgt, nt, T);
  return 0;
}

/* ----------------------------------------------------------------------- */
/* accumulate_clouds CropBox loop (accumulate_clouds.cpp:100-111)             */
/* ----------------------------------------------------------------------- */
size_t orc_crop_redundant(const orc_point* src, size_t ns, const orc_point* tgt, size_t nt, double radius,
                          uint8_t* removed) {
  const double cell = 2.0 * radius > 0 ? 2.0 * radius : 1.0;
  struct H { size_t operator()(const long long& k) const { return std::hash<long long>()(k); } };
  std::unordered_map<long long, std::vector<int>, H> grid;
  auto key = [&](long long a, long long b, long long c) { return (a * 73856093LL) ^ (b * 19349663LL) ^ (c * 83492791LL); };
  auto cellof = [&](double v) { return static_cast<long long>(std::floor(v / cell)); };
  for (size_t j = 0; j < nt; ++j) {
    if (!finite3(tgt[j])) continue;
    grid[key(cellof(tgt[j].x), cellof(tgt[j].y), cellof(tgt[j].z))].push_back(static_cast<int>(j));
  }
  /* PCL's CropBox (negative) drops a non-finite source point, and a box on a
   * non-finite target point holds every point (no NaN comparison says
   * "outside"): with any target point present, both remove. */
  bool tgt_bad = false;
  for (size_t j = 0; j < nt; ++j) tgt_bad = tgt_bad || !finite3(tgt[j]);
  size_t nrem = 0;
#pragma omp parallel for schedule(dynamic, 512) reduction(+ : nrem) num_threads(nthreads())
  for (long long i = 0; i < static_cast<long long>(ns); ++i) {
    removed[i] = 0;
    const orc_point& p = src[i];
    if (nt > 0 && (tgt_bad || !finite3(p))) { removed[i] = 1; ++nrem; continue; }
    if (!finite3(p)) continue;
    long long cx = cellof(p.x), cy = cellof(p.y), cz = cellof(p.z);
    bool hit = false;
    for (long long a = cx - 1; a <= cx + 1 && !hit; ++a)
      for (long long b = cy - 1; b <= cy + 1 && !hit; ++b)
        for (long long cc = cz - 1; cc <= cz + 1 && !hit; ++cc) {
          auto it = grid.find(key(a, b, cc));
          if (it == grid.end()) continue;
          for (int j : it->second) {
            const orc_point& q = tgt[j];
            float lx = static_cast<float>(q.x - radius), hx = static_cast<float>(q.x + radius);
            float ly = static_cast<float>(q.y - radius), hy = static_cast<float>(q.y + radius);
            float lz = static_cast<float>(q.z - radius), hz = static_cast<float>(q.z + radius);
            if (p.x >= lx && p.x <= hx && p.y >= ly && p.y <= hy && p.z >= lz && p.z <= hz) { hit = true; break; }
          }
        }
    if (hit) { removed[i] = 1; ++nrem; }
  }
  return nrem;
}

void orc_transform(const orc_point* in, size_t n, const float* m, orc_point* out) {
  for (size_t i = 0; i < n; ++i) {
    orc_point o = in[i];
    if (finite3(in[i])) {
      float a, b;
      a = m[0] * in[i].x; b = m[1] * in[i].y; a = a + b; b = m[2] * in[i].z; a = a + b; o.x = a + m[3];
      a = m[4] * in[i].x; b = m[5] * in[i].y; a = a + b; b = m[6] * in[i].z; a = a + b; o.y = a + m[7];
      a = m[8] * in[i].x; b = m[9] * in[i].y; a = a + b; b = m[10] * in[i].z; a = a + b; o.z = a + m[11];
      a = m[0] * in[i].normal_x; b = m[1] * in[i].normal_y; a = a + b; b = m[2] * in[i].normal_z; o.normal_x = a + b;
      a = m[4] * in[i].normal_x; b = m[5] * in[i].normal_y; a = a + b; b = m[6] * in[i].normal_z; o.normal_y = a + b;
      a = m[8] * in[i].normal_x; b = m[9] * in[i].normal_y; a = a + b; b = m[10] * in[i].normal_z; o.normal_z = a + b;
    }
    out[i] = o;
  }
}

void orc_centroid(const orc_point* in, size_t n, float* c) {
  float s[3] = {0, 0, 0};
  size_t cnt = 0;
  for (size_t i = 0; i < n; ++i) {
    if (!finite3(in[i])) continue;
    s[0] += in[i].x; s[1] += in[i].y; s[2] += in[i].z;
    ++cnt;
  }
  for (int a = 0; a < 3; ++a) c[a] = cnt ? s[a] / static_cast<float>(cnt) : 0.0f;
  c[3] = 1.0f;
}

void orc_svd3(const double* a, double* u, double* s, double* v) { svd3(a, u, s, v); }
void orc_eig3(const double* a, double* evals, double* evecs) { eig3_jacobi(a, evals, evecs); }

}  // extern "C"
