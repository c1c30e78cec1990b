// Synthetic capture pairs generated on the device: the training and
// evaluation data of the pose proposal, shaped like the turntable objects of
// the batched-ICP workload (a superquadric with extents 0.1-0.4 m, a block and
// two balls attached around it, seen by a camera at the origin looking down
// -z, 1 m away).
//
// Each view samples visible surface points: a candidate point on one of the
// parts (chosen in proportion to its approximate area) is kept when its
// outward normal faces the camera and it lies outside the other parts; the
// kept point gets Kinect-like depth noise along its ray,
// sigma = 1.5 mm (z / 1 m)^2.  The target view moves the object by a rotation
// about its vertical axis (uniform in +-yaw), a tilt (uniform in +-tilt) and a
// translation (uniform in +-translation per axis), so the ground-truth
// source-to-target transform is known exactly.  Everything is a hash of
// (seed, pair, view, point): the same seed gives the same clouds.
#include <cmath>

#include "lcr_internal.cuh"

namespace {

struct Part {
  int kind;          // 0 superquadric, 1 box, 2 ball
  float c[3];        // centre in the object frame
  float R[9];        // part orientation (row-major), object frame
  float a[3];        // semi-axes / half-extents / radius in a[0]
  float e1, e2;      // superquadric exponents
  float area;        // approximate surface area (sampling weight)
};

struct SynthObject {
  Part part[4];
  float cum[4];      // cumulative sampling weights, cum[3] = 1
  float Ps[12];      // object -> camera, source view (row-major 3x4)
  float Pt[12];      // object -> camera, target view
};

__host__ __device__ __forceinline__ uint64_t mix(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ float uni(uint64_t& s) {
  s = mix(s);
  return static_cast<float>(s >> 40) * (1.0f / 16777216.0f);
}

__device__ __forceinline__ float gauss(uint64_t& s) {
  const float u1 = fmaxf(uni(s), 1e-7f), u2 = uni(s);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}

__device__ void rot_y(float a, float* R) {
  const float c = cosf(a), s = sinf(a);
  const float m[9] = {c, 0, s, 0, 1, 0, -s, 0, c};
  for (int i = 0; i < 9; ++i) R[i] = m[i];
}

__device__ void rot_x(float a, float* R) {
  const float c = cosf(a), s = sinf(a);
  const float m[9] = {1, 0, 0, 0, c, -s, 0, s, c};
  for (int i = 0; i < 9; ++i) R[i] = m[i];
}

__device__ void mul3(const float* A, const float* B, float* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

// superquadric inside-outside function in the part frame (F <= 1 inside)
__device__ __forceinline__ float sq_f(const Part& p, float x, float y, float z) {
  const float ax = fabsf(x / p.a[0]) + 1e-12f, ay = fabsf(y / p.a[1]) + 1e-12f, az = fabsf(z / p.a[2]) + 1e-12f;
  const float A = powf(ax, 2.0f / p.e2) + powf(ay, 2.0f / p.e2);
  return powf(A, p.e2 / p.e1) + powf(az, 2.0f / p.e1);
}

__device__ __forceinline__ void to_part(const Part& p, const float* o, float* l) {
  const float d[3] = {o[0] - p.c[0], o[1] - p.c[1], o[2] - p.c[2]};
  for (int i = 0; i < 3; ++i) l[i] = p.R[i] * d[0] + p.R[3 + i] * d[1] + p.R[6 + i] * d[2];  // R^T d
}

__device__ bool inside(const Part& p, const float* o) {
  float l[3];
  to_part(p, o, l);
  if (p.kind == 0) return sq_f(p, l[0], l[1], l[2]) < 0.999f;
  if (p.kind == 1) return fabsf(l[0]) < p.a[0] * 0.999f && fabsf(l[1]) < p.a[1] * 0.999f && fabsf(l[2]) < p.a[2] * 0.999f;
  return l[0] * l[0] + l[1] * l[1] + l[2] * l[2] < p.a[0] * p.a[0] * 0.998f;
}

// A candidate point and outward normal on part p, object frame.
__device__ void surface_point(const Part& p, uint64_t& s, float* o, float* n) {
  float l[3], ln[3];
  if (p.kind == 2) {  // ball: uniform direction
    const float z = 2.0f * uni(s) - 1.0f, ph = 2.0f * uni(s), r = sqrtf(fmaxf(0.f, 1.0f - z * z));
    ln[0] = r * cospif(ph);
    ln[1] = r * sinpif(ph);
    ln[2] = z;
    for (int i = 0; i < 3; ++i) l[i] = p.a[0] * ln[i];
  } else if (p.kind == 1) {  // box: a face in proportion to its area, uniform on it
    const float w[3] = {p.a[1] * p.a[2], p.a[0] * p.a[2], p.a[0] * p.a[1]};
    float u = uni(s) * (w[0] + w[1] + w[2]);
    const int ax = u < w[0] ? 0 : (u < w[0] + w[1] ? 1 : 2);
    const float sg = uni(s) < 0.5f ? -1.f : 1.f;
    for (int i = 0; i < 3; ++i) {
      l[i] = (2.0f * uni(s) - 1.0f) * p.a[i];
      ln[i] = 0.f;
    }
    l[ax] = sg * p.a[ax];
    ln[ax] = sg;
  } else {  // superquadric: a uniform direction projected radially onto the surface
    const float z = 2.0f * uni(s) - 1.0f, ph = 2.0f * uni(s), r = sqrtf(fmaxf(0.f, 1.0f - z * z));
    const float d[3] = {r * cospif(ph), r * sinpif(ph), z};
    const float t = powf(sq_f(p, d[0], d[1], d[2]), -0.5f * p.e1);
    for (int i = 0; i < 3; ++i) l[i] = d[i] * t;
    const float ax = fabsf(l[0] / p.a[0]) + 1e-12f, ay = fabsf(l[1] / p.a[1]) + 1e-12f, az = fabsf(l[2] / p.a[2]) + 1e-12f;
    const float A = powf(ax, 2.0f / p.e2) + powf(ay, 2.0f / p.e2);
    const float k = powf(A, p.e2 / p.e1 - 1.0f);
    ln[0] = k * powf(ax, 2.0f / p.e2 - 1.0f) * copysignf(1.0f, l[0]) / p.a[0];
    ln[1] = k * powf(ay, 2.0f / p.e2 - 1.0f) * copysignf(1.0f, l[1]) / p.a[1];
    ln[2] = powf(az, 2.0f / p.e1 - 1.0f) * copysignf(1.0f, l[2]) / p.a[2];
    const float nn = rsqrtf(ln[0] * ln[0] + ln[1] * ln[1] + ln[2] * ln[2] + 1e-30f);
    for (int i = 0; i < 3; ++i) ln[i] *= nn;
  }
  for (int i = 0; i < 3; ++i) {
    o[i] = p.c[i] + p.R[3 * i] * l[0] + p.R[3 * i + 1] * l[1] + p.R[3 * i + 2] * l[2];
    n[i] = p.R[3 * i] * ln[0] + p.R[3 * i + 1] * ln[1] + p.R[3 * i + 2] * ln[2];
  }
}

// One thread per pair: the object and the two view poses.
// dist gives each pair's camera-to-object distance; else want gives the
// visible pixels wanted per view of a camera with focal lengths fx fy
// (fxfy = fx * fy): the distance at which the object's mean projected area
// (a quarter of its surface, Cauchy's formula for a convex body) covers that
// many pixels, within [0.4, 8] m; with neither, 1 m.
__global__ void k_synth_objects(uint64_t seed, int npairs, lcr_synth_params prm, SynthObject* __restrict__ objs,
                                float* __restrict__ T, const float* __restrict__ dist = nullptr,
                                const float* __restrict__ want = nullptr, float fxfy = 0.f) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= npairs) return;
  uint64_t s = mix(seed * 0x2545f4914f6cdd1dull + static_cast<uint64_t>(b) * 0x9e3779b97f4a7c15ull + 1);
  SynthObject o;
  const float d2r = 3.14159265358979f / 180.0f;
  // superquadric: semi-axes 0.05-0.2 m, exponents 0.3-1.5, random orientation
  Part& q = o.part[0];
  q.kind = 0;
  for (int i = 0; i < 3; ++i) {
    q.c[i] = 0.f;
    q.a[i] = 0.05f + 0.15f * uni(s);
  }
  q.e1 = 0.3f + 1.2f * uni(s);
  q.e2 = 0.3f + 1.2f * uni(s);
  float Ry[9], Rx[9];
  rot_y(2.0f * 3.14159265f * uni(s), Ry);
  rot_x((40.0f * uni(s) - 20.0f) * d2r, Rx);
  mul3(Ry, Rx, q.R);
  const float r = fmaxf(q.a[0], fmaxf(q.a[1], q.a[2]));
  {  // ellipsoid area (Knud Thomsen), scaled by how boxy the exponents make it
    const float pp = 1.6075f, ab = powf(q.a[0] * q.a[1], pp), ac = powf(q.a[0] * q.a[2], pp),
                bc = powf(q.a[1] * q.a[2], pp);
    q.area = 4.0f * 3.14159265f * powf((ab + ac + bc) / 3.0f, 1.0f / pp) * (1.0f + 0.3f * (2.0f - q.e1 - q.e2));
  }
  // a block and two balls around it, 120 degrees apart, at different heights
  const float a0 = 2.0f * 3.14159265f * uni(s);
  const float dy[3] = {-0.02f, 0.03f, -0.05f}, size[3] = {0.03f, 0.025f, 0.035f};
  for (int k = 1; k < 4; ++k) {
    Part& p = o.part[k];
    float side[9];
    rot_y(a0 + 2.0943951f * (k - 1), side);
    const float off = k == 1 ? r + 0.03f : r + 0.02f;
    const float lc[3] = {off, dy[k - 1], 0.f};
    for (int i = 0; i < 3; ++i) p.c[i] = side[3 * i] * lc[0] + side[3 * i + 1] * lc[1] + side[3 * i + 2] * lc[2];
    for (int i = 0; i < 9; ++i) p.R[i] = side[i];
    p.e1 = p.e2 = 1.f;
    if (k == 1) {
      p.kind = 1;
      p.a[0] = 0.03f;
      p.a[1] = 0.05f;
      p.a[2] = 0.02f;
      p.area = 8.0f * (p.a[0] * p.a[1] + p.a[1] * p.a[2] + p.a[0] * p.a[2]);
    } else {
      p.kind = 2;
      p.a[0] = p.a[1] = p.a[2] = size[k - 1];
      p.area = 4.0f * 3.14159265f * p.a[0] * p.a[0];
    }
  }
  float tot = 0.f;
  for (int k = 0; k < 4; ++k) tot += o.part[k].area;
  float acc = 0.f;
  for (int k = 0; k < 4; ++k) {
    acc += o.part[k].area / tot;
    o.cum[k] = acc;
  }
  o.cum[3] = 1.0f;
  // source view: the object turned about its vertical axis, in front of the camera
  float Rs[9];
  rot_y(2.0f * 3.14159265f * uni(s), Rs);
  float z = 1.0f;
  if (dist) z = dist[b];
  else if (want) z = fminf(fmaxf(sqrtf(0.25f * tot * fxfy / fmaxf(want[b], 1.f)), 0.4f), 8.0f);
  const float cs[3] = {0.f, 0.f, -z};
  // relative motion about the object centre: yaw, tilt, translation
  float Ryaw[9], Rtilt[9], Rrel[9], Rt[9];
  rot_y((2.0f * uni(s) - 1.0f) * prm.yaw_deg * d2r, Ryaw);
  rot_x((2.0f * uni(s) - 1.0f) * prm.tilt_deg * d2r, Rtilt);
  mul3(Rtilt, Ryaw, Rrel);
  mul3(Rrel, Rs, Rt);
  float tr[3];
  for (int i = 0; i < 3; ++i) tr[i] = (2.0f * uni(s) - 1.0f) * prm.translation;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      o.Ps[4 * i + j] = Rs[3 * i + j];
      o.Pt[4 * i + j] = Rt[3 * i + j];
    }
    o.Ps[4 * i + 3] = cs[i];
    o.Pt[4 * i + 3] = cs[i] + tr[i];
  }
  objs[b] = o;
  // ground truth source -> target: Pt Ps^-1 = [Rrel | c + tr - Rrel c]
  float* t = T + 16 * b;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) t[4 * i + j] = Rrel[3 * i + j];
    t[4 * i + 3] = cs[i] + tr[i] - (Rrel[3 * i] * cs[0] + Rrel[3 * i + 1] * cs[1] + Rrel[3 * i + 2] * cs[2]);
  }
  t[12] = t[13] = t[14] = 0.f;
  t[15] = 1.f;
}

// One thread per point of one view.
__global__ void k_synth_points(uint64_t seed, const SynthObject* __restrict__ objs, int npairs, int npts, int noise,
                               float4* const* __restrict__ xyz, float4* const* __restrict__ nrm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y, view = blockIdx.z;
  if (i >= npts || b >= npairs) return;
  const SynthObject& o = objs[b];
  const float* P = view == 0 ? o.Ps : o.Pt;
  uint64_t s = mix(seed ^ mix((static_cast<uint64_t>(b) << 33) ^ (static_cast<uint64_t>(view) << 32) ^
                              static_cast<uint64_t>(i)));
  float cam[3] = {0.f, 0.f, 0.f}, cn[3] = {0.f, 0.f, 1.f};
  bool found = false;
  for (int attempt = 0; attempt < 64 && !found; ++attempt) {
    const float u = uni(s);
    int k = 0;
    while (k < 3 && u > o.cum[k]) ++k;
    float ob[3], on[3];
    surface_point(o.part[k], s, ob, on);
    bool hidden = false;
    for (int j = 0; j < 4 && !hidden; ++j)
      if (j != k && inside(o.part[j], ob)) hidden = true;
    if (hidden) continue;
    float pc[3], pn[3];
    for (int r = 0; r < 3; ++r) {
      pc[r] = P[4 * r] * ob[0] + P[4 * r + 1] * ob[1] + P[4 * r + 2] * ob[2] + P[4 * r + 3];
      pn[r] = P[4 * r] * on[0] + P[4 * r + 1] * on[1] + P[4 * r + 2] * on[2];
    }
    if (pn[0] * pc[0] + pn[1] * pc[1] + pn[2] * pc[2] >= 0.f) continue;  // faces away from the camera
    for (int r = 0; r < 3; ++r) {
      cam[r] = pc[r];
      cn[r] = pn[r];
    }
    found = true;
  }
  if (noise && found) {
    const float z = -cam[2];
    const float dz = 0.0015f * z * z * gauss(s);
    const float f = (z + dz) / z;
    for (int r = 0; r < 3; ++r) cam[r] *= f;
  }
  const float nan = __int_as_float(0x7fc00000);
  xyz[2 * b + view][i] = found ? make_float4(cam[0], cam[1], cam[2], 0.f) : make_float4(nan, nan, nan, 0.f);
  nrm[2 * b + view][i] = make_float4(cn[0], cn[1], cn[2], 0.f);
}

// One block per cloud: RMS over its finite points of |Ta p - Tb p| (FP64).
__global__ void __launch_bounds__(256) k_rmse(const float4* const* __restrict__ xyz, const long long* __restrict__ n,
                                              const double* __restrict__ Ta, const double* __restrict__ Tb,
                                              double* __restrict__ out) {
  __shared__ double red[2][256];
  const int c = blockIdx.x;
  double A[12];
  for (int i = 0; i < 12; ++i) A[i] = Ta[16 * c + i] - Tb[16 * c + i];
  double s = 0.0, k = 0.0;
  for (long long i = threadIdx.x; i < n[c]; i += 256) {
    const float4 p = xyz[c][i];
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) continue;
    for (int r = 0; r < 3; ++r) {
      const double d = A[4 * r] * p.x + A[4 * r + 1] * p.y + A[4 * r + 2] * p.z + A[4 * r + 3];
      s += d * d;
    }
    k += 1.0;
  }
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = k;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[1][0] > 0 ? sqrt(red[0][0] / red[1][0]) : 0.0;
}

// ---------------------------------------------------------- depth images
// The same objects as a depth camera sees them.  Surface samples of each view
// (back-facing and covered ones dropped, as above) are splatted into a
// z-buffer, the smallest depth per pixel winning.  A sample gives the depth of
// its pixel's centre ray from its tangent plane, so planar faces render
// exactly and curved ones to second order; at grazing angles (or where the
// plane would move the depth by more than 2 cm) the sample's own depth is
// used.  Samples per view: spp per frontal pixel footprint (z/f)^2 of the
// object's whole area, so a visible pixel is missed with probability about
// exp(-spp/2) on a frontal surface and less where it is inclined.
struct RenderCam {
  int w, h;
  float fx, fy, cx, cy;
  float off;  // 0.5 for the Kinect v2 pixel-centre convention (kinect2.h:262-265), 0 otherwise
  float spp;
};

// Image v is view v&1 of pair v>>1 (views == null) or, on a turntable, pose
// views[v] (3x4 row-major object -> camera) of object 0.
__global__ void k_render_splat(uint64_t seed, const SynthObject* __restrict__ objs, RenderCam cam,
                               uint32_t* __restrict__ zbuf, const float* __restrict__ views = nullptr) {
  const int v = blockIdx.y, b = views ? 0 : v >> 1;
  const SynthObject& o = objs[b];
  const float* P = views ? views + 12 * v : ((v & 1) ? o.Pt : o.Ps);
  const float zc = fmaxf(-P[11], 0.05f);
  float area = 0.f;
  for (int k = 0; k < 4; ++k) area += o.part[k].area;
  const long long m = min(static_cast<long long>(cam.spp * area * cam.fx * cam.fy / (zc * zc)), 1ll << 28);
  const size_t plane = static_cast<size_t>(cam.w) * cam.h;
  uint32_t* zb = zbuf + static_cast<size_t>(v) * plane;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < m;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    uint64_t s = mix(seed ^ mix((static_cast<uint64_t>(v) << 36) ^ static_cast<uint64_t>(i) ^ 0x6a09e667f3bcc909ull));
    const float u = uni(s);
    int k = 0;
    while (k < 3 && u > o.cum[k]) ++k;
    float ob[3], on[3];
    surface_point(o.part[k], s, ob, on);
    bool hidden = false;
    for (int j = 0; j < 4 && !hidden; ++j)
      if (j != k && inside(o.part[j], ob)) hidden = true;
    if (hidden) continue;
    float pc[3], pn[3];
    for (int r = 0; r < 3; ++r) {
      pc[r] = P[4 * r] * ob[0] + P[4 * r + 1] * ob[1] + P[4 * r + 2] * ob[2] + P[4 * r + 3];
      pn[r] = P[4 * r] * on[0] + P[4 * r + 1] * on[1] + P[4 * r + 2] * on[2];
    }
    if (pn[0] * pc[0] + pn[1] * pc[1] + pn[2] * pc[2] >= 0.f) continue;  // faces away from the camera
    const float depth = -pc[2];
    if (!(depth > 0.05f)) continue;
    const int col = __float2int_rn(pc[0] * cam.fx / depth + cam.cx - cam.off);
    const int row = __float2int_rn(-pc[1] * cam.fy / depth + cam.cy - cam.off);
    if (col < 0 || col >= cam.w || row < 0 || row >= cam.h) continue;
    // the pixel centre's ray X = t d, d = ((col - cx + off)/fx, -(row - cy + off)/fy, -1): depth t
    const float dx = (static_cast<float>(col) - cam.cx + cam.off) / cam.fx;
    const float dy = -(static_cast<float>(row) - cam.cy + cam.off) / cam.fy;
    const float den = pn[0] * dx + pn[1] * dy - pn[2];
    float t = depth;
    if (fabsf(den) > 0.2f * sqrtf(dx * dx + dy * dy + 1.f)) {
      const float tp = (pn[0] * pc[0] + pn[1] * pc[1] + pn[2] * pc[2]) / den;
      if (fabsf(tp - depth) < 0.02f) t = tp;
    }
    atomicMin(zb + static_cast<size_t>(row) * cam.w + col, __float_as_uint(t));  // positive floats order as integers
  }
}

// z-buffer -> depth image: model 0 uint16 mm (rounded, saturated), else float
// mm; Kinect noise sigma = 1.5 mm (z / 1 m)^2 per pixel when noise is set;
// pixels without surface are 0.
__global__ void k_render_finish(uint64_t seed, const uint32_t* __restrict__ zbuf, int npix, int f32, int noise,
                                void* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const size_t at = static_cast<size_t>(blockIdx.y) * npix + p;
  const float z = __uint_as_float(zbuf[at]);
  float mm = 0.f;
  if (z < 1e30f) {
    mm = 1000.f * z;
    if (noise) {
      uint64_t s = mix(seed ^ mix((static_cast<uint64_t>(blockIdx.y) << 33) ^ static_cast<uint64_t>(p) ^
                                  0xbb67ae8584caa73bull));
      mm += 1.5f * z * z * gauss(s);
    }
  }
  if (f32) {
    static_cast<float*>(out)[at] = fmaxf(mm, 0.f);
  } else {
    static_cast<uint16_t*>(out)[at] = static_cast<uint16_t>(fminf(fmaxf(rintf(mm), 0.f), 65535.f));
  }
}

}  // namespace

void synth_depth(lcr_ctx* ctx, uint64_t seed, int npairs, const lcr_synth_params* prm, const lcr_render_params* cam,
                 const float* distance, const float* points, void* d_out, float* transforms) {
  if (npairs == 0) return;
  const size_t plane = static_cast<size_t>(cam->width) * cam->height;
  const size_t zbytes = plane * 4 * 2 * static_cast<size_t>(npairs);
  const size_t head = (npairs * sizeof(SynthObject) + npairs * 64 + npairs * 4 + 255) & ~static_cast<size_t>(255);
  char* d = static_cast<char*>(dev_alloc(ctx, head + zbytes));
  auto* objs = reinterpret_cast<SynthObject*>(d);
  auto* T = reinterpret_cast<float*>(d + npairs * sizeof(SynthObject));
  auto* dd = reinterpret_cast<float*>(d + npairs * sizeof(SynthObject) + npairs * 64);
  auto* zb = reinterpret_cast<uint32_t*>(d + head);
  const float* per_pair = distance ? distance : points;
  if (per_pair) CUDA_TRY(cudaMemcpyAsync(dd, per_pair, npairs * 4ull, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemsetAsync(zb, 0x7f, zbytes, ctx->stream));  // 0x7f7f7f7f: a float above any depth
  LCR_LAUNCH(ctx, k_synth_objects, (npairs + 127) / 128, 128, 0, seed, npairs, *prm, objs, T,
             distance ? static_cast<const float*>(dd) : nullptr, points ? static_cast<const float*>(dd) : nullptr,
             static_cast<float>(cam->fx * cam->fy));
  RenderCam rc;
  rc.w = cam->width;
  rc.h = cam->height;
  rc.fx = static_cast<float>(cam->fx);
  rc.fy = static_cast<float>(cam->fy);
  rc.cx = static_cast<float>(cam->cx);
  rc.cy = static_cast<float>(cam->cy);
  rc.off = cam->model == LCR_DEPTH_KINECT_V2 ? 0.5f : 0.f;
  rc.spp = cam->samples_per_pixel > 0 ? cam->samples_per_pixel : 6.f;
  LCR_LAUNCH(ctx, k_render_splat, dim3(64, 2 * npairs), 256, 0, seed, objs, rc, zb);
  const int f32 = cam->model == LCR_DEPTH_KINECT_V1 ? 0 : 1;
  LCR_LAUNCH(ctx, k_render_finish, dim3(static_cast<unsigned>((plane + 255) / 256), 2 * npairs), 256, 0, seed, zb,
             static_cast<int>(plane), f32, prm->noise, d_out);
  CUDA_TRY(cudaMemcpyAsync(transforms, T, npairs * 64ull, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  dev_free(ctx, d);
}

// The turntable poses: view v turns the object by v * step about its vertical
// axis through its centre, from the object's own source pose (pair 0 of the
// seed); poses[v] = object -> camera, 4x4 row-major.
__global__ void k_turntable_poses(const SynthObject* __restrict__ objs, int views, float step_rad,
                                  float* __restrict__ P12, float* __restrict__ poses) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= views) return;
  const float* Ps = objs[0].Ps;
  float Rv[9];
  rot_y(step_rad * static_cast<float>(v), Rv);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) {
      const float r = Rv[3 * i] * Ps[j] + Rv[3 * i + 1] * Ps[4 + j] + Rv[3 * i + 2] * Ps[8 + j];
      P12[12 * v + 4 * i + j] = r;
      poses[16 * v + 4 * i + j] = r;
    }
    P12[12 * v + 4 * i + 3] = Ps[4 * i + 3];
    poses[16 * v + 4 * i + 3] = Ps[4 * i + 3];
  }
  poses[16 * v + 12] = poses[16 * v + 13] = poses[16 * v + 14] = 0.f;
  poses[16 * v + 15] = 1.f;
}

void synth_turntable(lcr_ctx* ctx, uint64_t seed, int views, float step_deg, const lcr_render_params* cam,
                     float distance, int noise, void* d_out, float* poses) {
  if (views == 0) return;
  const size_t plane = static_cast<size_t>(cam->width) * cam->height;
  const size_t zbytes = plane * 4 * static_cast<size_t>(views);
  const size_t head = (sizeof(SynthObject) + 64 + 4 + views * (48 + 64) + 255) & ~static_cast<size_t>(255);
  char* d = static_cast<char*>(dev_alloc(ctx, head + zbytes));
  auto* objs = reinterpret_cast<SynthObject*>(d);
  auto* T = reinterpret_cast<float*>(d + sizeof(SynthObject));
  auto* dd = reinterpret_cast<float*>(d + sizeof(SynthObject) + 64);
  auto* P12 = reinterpret_cast<float*>(d + sizeof(SynthObject) + 68);
  auto* P16 = P12 + 12 * views;
  auto* zb = reinterpret_cast<uint32_t*>(d + head);
  CUDA_TRY(cudaMemcpyAsync(dd, &distance, 4, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemsetAsync(zb, 0x7f, zbytes, ctx->stream));
  lcr_synth_params prm{0.f, 0.f, 0.f, noise};
  LCR_LAUNCH(ctx, k_synth_objects, 1, 32, 0, seed, 1, prm, objs, T, static_cast<const float*>(dd),
             static_cast<const float*>(nullptr), 0.f);
  LCR_LAUNCH(ctx, k_turntable_poses, (views + 63) / 64, 64, 0, objs, views,
             step_deg * 3.14159265358979f / 180.0f, P12, P16);
  RenderCam rc;
  rc.w = cam->width;
  rc.h = cam->height;
  rc.fx = static_cast<float>(cam->fx);
  rc.fy = static_cast<float>(cam->fy);
  rc.cx = static_cast<float>(cam->cx);
  rc.cy = static_cast<float>(cam->cy);
  rc.off = cam->model == LCR_DEPTH_KINECT_V2 ? 0.5f : 0.f;
  rc.spp = cam->samples_per_pixel > 0 ? cam->samples_per_pixel : 6.f;
  LCR_LAUNCH(ctx, k_render_splat, dim3(64, views), 256, 0, seed, objs, rc, zb, static_cast<const float*>(P12));
  const int f32 = cam->model == LCR_DEPTH_KINECT_V1 ? 0 : 1;
  LCR_LAUNCH(ctx, k_render_finish, dim3(static_cast<unsigned>((plane + 255) / 256), views), 256, 0, seed, zb,
             static_cast<int>(plane), f32, noise, d_out);
  CUDA_TRY(cudaMemcpyAsync(poses, P16, views * 64ull, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  dev_free(ctx, d);
}

void rmse_batch(lcr_ctx* ctx, const lcr_cloud* const* clouds, int n, const double* Ta, const double* Tb,
                double* out) {
  if (n == 0) return;
  const size_t bytes = n * (sizeof(float4*) + 8 + 128 + 128 + 8);
  char* d = static_cast<char*>(dev_alloc(ctx, bytes));
  auto* dp = reinterpret_cast<const float4**>(d);
  auto* dn = reinterpret_cast<long long*>(d + n * sizeof(float4*));
  auto* da = reinterpret_cast<double*>(d + n * (sizeof(float4*) + 8));
  auto* db = da + 16 * static_cast<size_t>(n);
  auto* dout = db + 16 * static_cast<size_t>(n);
  std::vector<const float4*> hp(n);
  std::vector<long long> hn(n);
  for (int i = 0; i < n; ++i) {
    hp[i] = clouds[i]->xyz;
    hn[i] = static_cast<long long>(clouds[i]->n);
  }
  CUDA_TRY(cudaMemcpyAsync(dp, hp.data(), n * sizeof(float4*), cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(dn, hn.data(), n * 8ull, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(da, Ta, n * 128ull, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(db, Tb, n * 128ull, cudaMemcpyHostToDevice, ctx->stream));
  LCR_LAUNCH(ctx, k_rmse, n, 256, 0, dp, dn, da, db, dout);
  CUDA_TRY(cudaMemcpyAsync(out, dout, n * 8ull, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  dev_free(ctx, d);
}

void synth_pairs(lcr_ctx* ctx, uint64_t seed, int npairs, int npts, const lcr_synth_params* prm, lcr_cloud** src,
                 lcr_cloud** tgt, float* transforms) {
  if (npairs == 0) return;
  const size_t ptr_bytes = 2 * sizeof(float4*) * 2 * static_cast<size_t>(npairs);
  char* d = static_cast<char*>(dev_alloc(ctx, npairs * sizeof(SynthObject) + npairs * 64 + ptr_bytes));
  auto* objs = reinterpret_cast<SynthObject*>(d);
  auto* T = reinterpret_cast<float*>(d + npairs * sizeof(SynthObject));
  auto* ptrs = reinterpret_cast<float4**>(d + npairs * sizeof(SynthObject) + npairs * 64);
  std::vector<float4*> hp(4 * static_cast<size_t>(npairs));
  for (int b = 0; b < npairs; ++b) {
    src[b] = cloud_alloc(ctx, npts);
    tgt[b] = cloud_alloc(ctx, npts);
    hp[2 * b] = src[b]->xyz;
    hp[2 * b + 1] = tgt[b]->xyz;
    hp[2 * npairs + 2 * b] = src[b]->nrm;
    hp[2 * npairs + 2 * b + 1] = tgt[b]->nrm;
    CUDA_TRY(cudaMemsetAsync(src[b]->rgb, 0xff, npts * 4ull, ctx->stream));
    CUDA_TRY(cudaMemsetAsync(tgt[b]->rgb, 0xff, npts * 4ull, ctx->stream));
  }
  CUDA_TRY(cudaMemcpyAsync(ptrs, hp.data(), ptr_bytes, cudaMemcpyHostToDevice, ctx->stream));
  LCR_LAUNCH(ctx, k_synth_objects, (npairs + 127) / 128, 128, 0, seed, npairs, *prm, objs, T);
  const dim3 grid((npts + 255) / 256, npairs, 2);
  LCR_LAUNCH(ctx, k_synth_points, grid, 256, 0, seed, objs, npairs, npts, prm->noise, ptrs, ptrs + 2 * npairs);
  CUDA_TRY(cudaMemcpyAsync(transforms, T, npairs * 64ull, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  dev_free(ctx, d);
}
