// Depth-image -> point-cloud path: burst fusion (zero-eliminated mean) and the
// Kinect v1 / v2 back-projections, reproducing the reference's arithmetic with
// explicit IEEE intrinsics (no FMA contraction) so results are bit-exact.
#include <algorithm>
#include <mutex>

#include "lcr_internal.cuh"

namespace {

struct BP {
  int w, h;
  double ifx, ify, cx, cy;  // V1: 1/fx, 1/fy in double as the reference computes them
  float fxf, fyf, cxf, cyf; // V2: libfreenect2's float intrinsics
  double dmin, dmax, scale;
  float scalef;
  int left, right, top, bottom;
  int normals;
  uint32_t rgb;
};

// super_resolution.cpp:295-315: mean of the non-zero samples in double, returned
// as float, then converted to uint16 with round-half-even and saturation.  With
// no sample the reference's 0/0 NaN saturates to 0.
__global__ void k_fuse_u16(const uint16_t* __restrict__ frames, int F, size_t npix, uint16_t* __restrict__ out) {
  const size_t p = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  uint32_t sum = 0, cnt = 0;
  for (int f = 0; f < F; ++f) {
    const uint32_t v = frames[static_cast<size_t>(f) * npix + p];
    if (v) { sum += v; ++cnt; }
  }
  uint16_t r = 0;
  if (cnt) {
    const float m = __double2float_rn(__ddiv_rn(static_cast<double>(sum), static_cast<double>(cnt)));
    const int ri = __float2int_rn(m);
    r = static_cast<uint16_t>(ri <= 0 ? 0 : (ri >= 65535 ? 65535 : ri));
  }
  out[p] = r;
}

// super_resolution_kv2.cpp:287-303 (guarded: an empty pixel stays 0).
__global__ void k_fuse_f32(const float* __restrict__ frames, int F, size_t npix, float* __restrict__ out) {
  const size_t p = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  double sum = 0.0;
  uint32_t cnt = 0;
  for (int f = 0; f < F; ++f) {
    const float v = frames[static_cast<size_t>(f) * npix + p];
    if (v > 0.f) { sum = __dadd_rn(sum, static_cast<double>(v)); ++cnt; }
  }
  out[p] = cnt ? __double2float_rn(__ddiv_rn(sum, static_cast<double>(cnt))) : 0.f;
}

// The pinhole models keep a pixel with a depth in [dmin, dmax] inside the
// window: uint16 depth (Kinect v1, depth_capture.cpp, super_resolution.cpp
// save_ply) or float depth (super_resolution_kv2.cpp save_ply :25-118).
template <typename T>
__device__ __forceinline__ bool keep_v1(const BP& b, int i, int j, T z) {
  return z != 0 && static_cast<double>(z) >= b.dmin && static_cast<double>(z) <= b.dmax && i >= b.top &&
         i <= b.bottom && j >= b.left && j <= b.right;
}

template <typename T>
__global__ void k_flags_v1(const T* __restrict__ depth, BP b, uint8_t* __restrict__ flags) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= b.w * b.h) return;
  const int i = p / b.w, j = p - i * b.w;
  flags[p] = keep_v1(b, i, j, depth[p]) ? 1 : 0;
}

// depth_capture.cpp:231-265 (rows are the "x" direction of the gradient).
__device__ __forceinline__ float3 image_normal(const uint16_t* __restrict__ d, int w, int h, int i, int j) {
  const int c = d[static_cast<size_t>(i) * w + j];
  int right = 0, left = 0, down = 0, up = 0;
  if (i > 0 && j > 0 && i < h - 1 && j < w - 1) {
    right = d[static_cast<size_t>(i + 1) * w + j];
    left = d[static_cast<size_t>(i - 1) * w + j];
    down = d[static_cast<size_t>(i) * w + j + 1];
    up = d[static_cast<size_t>(i) * w + j - 1];
  }
  if (abs(c - right) > 20) right = 0;
  if (abs(c - left) > 20) left = 0;
  if (abs(c - down) > 20) down = 0;
  if (abs(c - up) > 20) up = 0;
  const double dzdx = __ddiv_rn(static_cast<double>(right - left), 2.0);
  const double dzdy = __ddiv_rn(static_cast<double>(down - up), 2.0);
  const double d0 = -dzdx, d1 = -dzdy, d2 = 1.0;
  double s = __dmul_rn(d0, d0);
  s = __dadd_rn(s, __dmul_rn(d1, d1));
  s = __dadd_rn(s, __dmul_rn(d2, d2));
  const double nv = __dsqrt_rn(s);
  const double inv = nv != 0.0 ? __ddiv_rn(1.0, nv) : 0.0;
  return make_float3(__double2float_rn(__dmul_rn(d0, inv)), __double2float_rn(__dmul_rn(d1, inv)),
                     __double2float_rn(__dmul_rn(d2, inv)));
}

// super_resolution_kv2.cpp:33-62, the same rule on float depth: the
// differences and the threshold test are FP32, the slopes FP64.
__device__ __forceinline__ float3 image_normal(const float* __restrict__ d, int w, int h, int i, int j) {
  const float c = d[static_cast<size_t>(i) * w + j];
  float right = 0.f, left = 0.f, down = 0.f, up = 0.f;
  if (i > 0 && j > 0 && i < h - 1 && j < w - 1) {
    right = d[static_cast<size_t>(i + 1) * w + j];
    left = d[static_cast<size_t>(i - 1) * w + j];
    down = d[static_cast<size_t>(i) * w + j + 1];
    up = d[static_cast<size_t>(i) * w + j - 1];
  }
  if (fabsf(__fsub_rn(c, right)) > 20.f) right = 0.f;
  if (fabsf(__fsub_rn(c, left)) > 20.f) left = 0.f;
  if (fabsf(__fsub_rn(c, down)) > 20.f) down = 0.f;
  if (fabsf(__fsub_rn(c, up)) > 20.f) up = 0.f;
  const double dzdx = __ddiv_rn(static_cast<double>(__fsub_rn(right, left)), 2.0);
  const double dzdy = __ddiv_rn(static_cast<double>(__fsub_rn(down, up)), 2.0);
  const double d0 = -dzdx, d1 = -dzdy, d2 = 1.0;
  double s = __dmul_rn(d0, d0);
  s = __dadd_rn(s, __dmul_rn(d1, d1));
  s = __dadd_rn(s, __dmul_rn(d2, d2));
  const double nv = __dsqrt_rn(s);
  const double inv = nv != 0.0 ? __ddiv_rn(1.0, nv) : 0.0;
  return make_float3(__double2float_rn(__dmul_rn(d0, inv)), __double2float_rn(__dmul_rn(d1, inv)),
                     __double2float_rn(__dmul_rn(d2, inv)));
}

// depth_capture.cpp:294-308: x = z*(j-cx)*(1/fx), y = -z*(i-cy)*(1/fy), z' = -z in
// double, times `scale`, rounded once to float (the same for float depth,
// super_resolution_kv2.cpp:96-106).
template <typename T>
__global__ void k_emit_v1(const T* __restrict__ depth, BP b, const uint32_t* __restrict__ idx, int n,
                          float4* __restrict__ xyz, float4* __restrict__ nrm, uint32_t* __restrict__ rgb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int p = static_cast<int>(idx[k]);
  const int i = p / b.w, j = p - i * b.w;
  const double z = static_cast<double>(depth[p]);
  const double vx = __dmul_rn(__dmul_rn(z, __dsub_rn(static_cast<double>(j), b.cx)), b.ifx);
  const double vy = __dmul_rn(__dmul_rn(-z, __dsub_rn(static_cast<double>(i), b.cy)), b.ify);
  const double vz = -z;
  xyz[k] = make_float4(__double2float_rn(__dmul_rn(vx, b.scale)), __double2float_rn(__dmul_rn(vy, b.scale)),
                       __double2float_rn(__dmul_rn(vz, b.scale)), 0.f);
  float3 nn = make_float3(0.f, 0.f, 0.f);
  if (b.normals) nn = image_normal(depth, b.w, b.h, i, j);
  nrm[k] = make_float4(nn.x, nn.y, nn.z, 0.f);
  rgb[k] = b.rgb;
}

// kinect2.h:169-187 + depth_capture_kv2.cpp:233-245 for one pixel.  Returns
// whether the point survives; p receives the (unscaled) point.
__device__ __forceinline__ bool point_v2(const BP& b, const float* __restrict__ depth, int yy, int xx, float3& p) {
  const float dv = __fdiv_rn(depth[static_cast<size_t>(yy) * b.w + xx], 1000.0f);
  if (isnan(dv) || static_cast<double>(fabsf(dv)) < 0.0001) return false;
  const float cm =
      __double2float_rn(__ddiv_rn(__dadd_rn(static_cast<double>(__fsub_rn(static_cast<float>(xx), b.cxf)), 0.5),
                                  static_cast<double>(b.fxf)));
  const float rm =
      __double2float_rn(__ddiv_rn(__dadd_rn(static_cast<double>(__fsub_rn(static_cast<float>(yy), b.cyf)), 0.5),
                                  static_cast<double>(b.fyf)));
  const float px = __fmul_rn(cm, dv);
  const float py = -__fmul_rn(rm, dv);
  const float pz = -dv;
  const float X = __double2float_rn(__dadd_rn(
      __dsub_rn(static_cast<double>(__fmul_rn(__fdiv_rn(px, -pz), b.fxf)), 0.5), static_cast<double>(b.cxf)));
  const float Y = __double2float_rn(__dadd_rn(
      __dsub_rn(static_cast<double>(__fmul_rn(__fdiv_rn(-py, -pz), b.fyf)), 0.5), static_cast<double>(b.cyf)));
  const float D = __double2float_rn(__dmul_rn(static_cast<double>(-pz), 1000.0));
  if (!(D != 0.f && D >= b.dmin && D <= b.dmax && Y >= static_cast<float>(b.top) && Y <= static_cast<float>(b.bottom) &&
        X >= static_cast<float>(b.left) && X <= static_cast<float>(b.right)))
    return false;
  p = make_float3(px, py, pz);
  return true;
}

__global__ void k_flags_v2(const float* __restrict__ depth, BP b, uint8_t* __restrict__ flags) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= b.w * b.h) return;
  const int yy = p / b.w, xx = p - yy * b.w;
  float3 q;
  flags[p] = point_v2(b, depth, yy, xx, q) ? 1 : 0;
}

__global__ void k_emit_v2(const float* __restrict__ depth, BP b, const uint32_t* __restrict__ idx, int n,
                          float4* __restrict__ xyz, float4* __restrict__ nrm, uint32_t* __restrict__ rgb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int p = static_cast<int>(idx[k]);
  const int yy = p / b.w, xx = p - yy * b.w;
  float3 q = make_float3(0.f, 0.f, 0.f);
  point_v2(b, depth, yy, xx, q);
  xyz[k] = make_float4(__fmul_rn(b.scalef, q.x), __fmul_rn(b.scalef, q.y), __fmul_rn(b.scalef, q.z), 0.f);
  nrm[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  rgb[k] = b.rgb;
}

BP make_bp(const lcr_depth_params* p) {
  BP b;
  b.w = p->width;
  b.h = p->height;
  b.ifx = 1 / p->fx;
  b.ify = 1 / p->fy;
  b.cx = p->cx;
  b.cy = p->cy;
  b.fxf = static_cast<float>(p->fx);
  b.fyf = static_cast<float>(p->fy);
  b.cxf = static_cast<float>(p->cx);
  b.cyf = static_cast<float>(p->cy);
  b.dmin = p->depth_min;
  b.dmax = p->depth_max;
  b.scale = p->scale;
  b.scalef = static_cast<float>(p->scale);
  b.left = p->roi_left;
  b.right = p->roi_right;
  b.top = p->roi_top;
  b.bottom = p->roi_bottom;
  b.normals = p->normals;
  b.rgb = static_cast<uint32_t>(p->b) | (static_cast<uint32_t>(p->g) << 8) | (static_cast<uint32_t>(p->r) << 16);
  return b;
}

}  // namespace

void burst_fuse_run(lcr_ctx* ctx, const void* d_frames, const lcr_depth_params* p, void* d_out) {
  const size_t npix = static_cast<size_t>(p->width) * p->height;
  const unsigned grid = static_cast<unsigned>((npix + 255) / 256);
  if (p->model == LCR_DEPTH_KINECT_V1)
    LCR_LAUNCH(ctx, k_fuse_u16, grid, 256, 0, static_cast<const uint16_t*>(d_frames), p->frames, npix,
               static_cast<uint16_t*>(d_out));
  else
    LCR_LAUNCH(ctx, k_fuse_f32, grid, 256, 0, static_cast<const float*>(d_frames), p->frames, npix,
               static_cast<float*>(d_out));
}

int backproject_run(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p, lcr_cloud** out) {
  const int npix = p->width * p->height;
  const BP b = make_bp(p);
  const size_t esz = p->model == LCR_DEPTH_KINECT_V1 ? 2 : 4;
  void* fused = nullptr;
  const void* depth = d_depth;
  if (p->frames > 1) {
    fused = dev_alloc(ctx, npix * esz);
    burst_fuse_run(ctx, d_depth, p, fused);
    depth = fused;
  }
  uint8_t* flags = static_cast<uint8_t*>(dev_alloc(ctx, npix));
  uint32_t* idx = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * npix));
  const unsigned grid = (npix + 255) / 256;
  if (p->model == LCR_DEPTH_KINECT_V1)
    LCR_LAUNCH(ctx, k_flags_v1<uint16_t>, grid, 256, 0, static_cast<const uint16_t*>(depth), b, flags);
  else if (p->model == LCR_DEPTH_PINHOLE_F32)
    LCR_LAUNCH(ctx, k_flags_v1<float>, grid, 256, 0, static_cast<const float*>(depth), b, flags);
  else
    LCR_LAUNCH(ctx, k_flags_v2, grid, 256, 0, static_cast<const float*>(depth), b, flags);
  const int n = compact_flags(ctx, flags, npix, idx);
  lcr_cloud* c = cloud_alloc(ctx, n);
  if (n > 0) {
    const unsigned eg = (n + 255) / 256;
    if (p->model == LCR_DEPTH_KINECT_V1)
      LCR_LAUNCH(ctx, k_emit_v1<uint16_t>, eg, 256, 0, static_cast<const uint16_t*>(depth), b, idx, n, c->xyz, c->nrm,
                 c->rgb);
    else if (p->model == LCR_DEPTH_PINHOLE_F32)
      LCR_LAUNCH(ctx, k_emit_v1<float>, eg, 256, 0, static_cast<const float*>(depth), b, idx, n, c->xyz, c->nrm,
                 c->rgb);
    else
      LCR_LAUNCH(ctx, k_emit_v2, eg, 256, 0, static_cast<const float*>(depth), b, idx, n, c->xyz, c->nrm, c->rgb);
  }
  dev_free(ctx, flags);
  dev_free(ctx, idx);
  dev_free(ctx, fused);
  *out = c;
  return n;
}

// ------------------------------------------------- allocation-free variant
// lcr_backproject_into: the same points as backproject_run, written as
// lcr_point records into caller-owned device memory, with its scratch in one
// static device buffer (the fused image of a burst and the per-block counts of
// the compaction) instead of allocations.
namespace {

constexpr int kIntoMaxPixels = 640 * 480;                   // the largest image the scratch holds
constexpr int kIntoBlock = 256;                             // pixels per compaction block
constexpr int kIntoMaxBlocks = kIntoMaxPixels / kIntoBlock;  // 1200
constexpr size_t kIntoFusedBytes = static_cast<size_t>(kIntoMaxPixels) * 4;  // float (v2) or uint16 (v1)
constexpr size_t kIntoScratchBytes = kIntoFusedBytes + static_cast<size_t>(kIntoMaxBlocks) * 4;
constexpr int kIntoMaxDevices = 64;

__device__ __align__(256) unsigned char g_into_scratch[kIntoScratchBytes];

std::mutex g_into_mutex;
void* g_into_addr[kIntoMaxDevices] = {};

// Device address of the scratch on `device` (looked up once per device).
unsigned char* into_scratch(int device) {
  if (device < 0 || device >= kIntoMaxDevices)
    LCR_THROW(LCR_ERR_INVALID_ARG, "lcr_backproject_into supports devices 0..%d", kIntoMaxDevices - 1);
  std::lock_guard<std::mutex> lock(g_into_mutex);
  if (!g_into_addr[device]) {
    void* a = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&a, g_into_scratch);
    if (e != cudaSuccess) LCR_THROW(LCR_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_into_addr[device] = a;
  }
  return static_cast<unsigned char*>(g_into_addr[device]);
}

// Kept pixel test of one pixel, and its record, for each camera model M
// (LCR_DEPTH_KINECT_V1, LCR_DEPTH_KINECT_V2, LCR_DEPTH_PINHOLE_F32).
template <int M>
__device__ __forceinline__ bool into_keep(const void* depth, const BP& b, int p) {
  const int i = p / b.w, j = p - i * b.w;
  if (M == LCR_DEPTH_KINECT_V1) return keep_v1(b, i, j, static_cast<const uint16_t*>(depth)[p]);
  if (M == LCR_DEPTH_PINHOLE_F32) return keep_v1(b, i, j, static_cast<const float*>(depth)[p]);
  float3 q;
  return point_v2(b, static_cast<const float*>(depth), i, j, q);
}

template <int M>
__device__ __forceinline__ void into_record(const void* depth, const BP& b, int p, float4* __restrict__ rec) {
  const int i = p / b.w, j = p - i * b.w;
  float4 xyz;
  float3 nn = make_float3(0.f, 0.f, 0.f);
  if (M != LCR_DEPTH_KINECT_V2) {
    // depth_capture.cpp:294-308, as k_emit_v1
    const double z = M == LCR_DEPTH_KINECT_V1 ? static_cast<double>(static_cast<const uint16_t*>(depth)[p])
                                              : static_cast<double>(static_cast<const float*>(depth)[p]);
    const double vx = __dmul_rn(__dmul_rn(z, __dsub_rn(static_cast<double>(j), b.cx)), b.ifx);
    const double vy = __dmul_rn(__dmul_rn(-z, __dsub_rn(static_cast<double>(i), b.cy)), b.ify);
    const double vz = -z;
    xyz = make_float4(__double2float_rn(__dmul_rn(vx, b.scale)), __double2float_rn(__dmul_rn(vy, b.scale)),
                      __double2float_rn(__dmul_rn(vz, b.scale)), 1.f);
    if (b.normals) {
      if (M == LCR_DEPTH_KINECT_V1)
        nn = image_normal(static_cast<const uint16_t*>(depth), b.w, b.h, i, j);
      else
        nn = image_normal(static_cast<const float*>(depth), b.w, b.h, i, j);
    }
  } else {
    float3 q = make_float3(0.f, 0.f, 0.f);
    point_v2(b, static_cast<const float*>(depth), i, j, q);
    xyz = make_float4(__fmul_rn(b.scalef, q.x), __fmul_rn(b.scalef, q.y), __fmul_rn(b.scalef, q.z), 1.f);
  }
  // lcr_point: {x y z 1} {nx ny nz 0} {rgba curvature 0 0}
  rec[0] = xyz;
  rec[1] = make_float4(nn.x, nn.y, nn.z, 0.f);
  rec[2] = make_float4(__uint_as_float(b.rgb), 0.f, 0.f, 0.f);
}

template <int M>
__global__ void __launch_bounds__(kIntoBlock) k_into_count(const void* depth, BP b, uint32_t* __restrict__ counts) {
  const int p = blockIdx.x * kIntoBlock + threadIdx.x;
  const bool k = p < b.w * b.h && into_keep<M>(depth, b, p);
  const int c = __syncthreads_count(k);
  if (threadIdx.x == 0) counts[blockIdx.x] = static_cast<uint32_t>(c);
}

// Exclusive scan of the block counts in place (one block; nblk <= 1200) and
// the total into *count.
__global__ void __launch_bounds__(1024) k_into_scan(uint32_t* __restrict__ counts, int nblk, uint32_t* count) {
  __shared__ uint32_t s_w[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  uint32_t carry = 0;
  for (int base = 0; base < nblk; base += 1024) {
    const int i = base + t;
    const uint32_t v = i < nblk ? counts[i] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(LCR_FULL, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) s_w[w] = incl;
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (int k = 0; k < 32; ++k) {
      before += k < w ? s_w[k] : 0u;
      all += s_w[k];
    }
    if (i < nblk) counts[i] = carry + before + incl - v;
    carry += all;
    __syncthreads();
  }
  if (t == 0) *count = carry;
}

// Each block recomputes its pixels' keep flags, ranks them in pixel order and
// writes their records from its scanned offset; nothing past `capacity`.
template <int M>
__global__ void __launch_bounds__(kIntoBlock) k_into_emit(const void* depth, BP b, const uint32_t* __restrict__ offs,
                                                          float4* __restrict__ rec, size_t capacity) {
  __shared__ uint32_t s_w[kIntoBlock / 32];
  const int p = blockIdx.x * kIntoBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool k = p < b.w * b.h && into_keep<M>(depth, b, p);
  const unsigned m = __ballot_sync(LCR_FULL, k);
  if (lane == 0) s_w[w] = __popc(m);
  __syncthreads();
  uint32_t before = 0;
  for (int j = 0; j < w; ++j) before += s_w[j];
  if (!k) return;
  const size_t pos = static_cast<size_t>(offs[blockIdx.x]) + before + __popc(m & ((1u << lane) - 1u));
  if (pos < capacity) into_record<M>(depth, b, p, rec + 3 * pos);
}

}  // namespace

void backproject_into_run(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p, lcr_point* d_points,
                          size_t capacity, uint32_t* d_count) {
  const long long npix = static_cast<long long>(p->width) * p->height;
  if (npix > kIntoMaxPixels)
    LCR_THROW(LCR_ERR_INVALID_ARG, "lcr_backproject_into: %dx%d = %lld pixels exceeds its %d-pixel scratch (640x480)",
              p->width, p->height, npix, kIntoMaxPixels);
  unsigned char* scratch = into_scratch(ctx->device);
  void* fused = scratch;
  uint32_t* counts = reinterpret_cast<uint32_t*>(scratch + kIntoFusedBytes);
  const BP b = make_bp(p);
  const void* depth = d_depth;
  if (p->frames > 1) {
    burst_fuse_run(ctx, d_depth, p, fused);
    depth = fused;
  }
  const int nblk = static_cast<int>((npix + kIntoBlock - 1) / kIntoBlock);
  float4* rec = reinterpret_cast<float4*>(d_points);
  if (p->model == LCR_DEPTH_KINECT_V1) {
    LCR_LAUNCH(ctx, k_into_count<LCR_DEPTH_KINECT_V1>, nblk, kIntoBlock, 0, depth, b, counts);
    LCR_LAUNCH(ctx, k_into_scan, 1, 1024, 0, counts, nblk, d_count);
    LCR_LAUNCH(ctx, k_into_emit<LCR_DEPTH_KINECT_V1>, nblk, kIntoBlock, 0, depth, b, counts, rec, capacity);
  } else if (p->model == LCR_DEPTH_PINHOLE_F32) {
    LCR_LAUNCH(ctx, k_into_count<LCR_DEPTH_PINHOLE_F32>, nblk, kIntoBlock, 0, depth, b, counts);
    LCR_LAUNCH(ctx, k_into_scan, 1, 1024, 0, counts, nblk, d_count);
    LCR_LAUNCH(ctx, k_into_emit<LCR_DEPTH_PINHOLE_F32>, nblk, kIntoBlock, 0, depth, b, counts, rec, capacity);
  } else {
    LCR_LAUNCH(ctx, k_into_count<LCR_DEPTH_KINECT_V2>, nblk, kIntoBlock, 0, depth, b, counts);
    LCR_LAUNCH(ctx, k_into_scan, 1, 1024, 0, counts, nblk, d_count);
    LCR_LAUNCH(ctx, k_into_emit<LCR_DEPTH_KINECT_V2>, nblk, kIntoBlock, 0, depth, b, counts, rec, capacity);
  }
}
