// Internal declarations shared by the liblcr CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "../../include/lcr.h"

#define LCR_FULL 0xffffffffu

// ---------------------------------------------------------------- errors
struct LcrError {
  lcr_status st;
  std::string msg;
};

// Throwing inside the library, caught at the C ABI boundary (api.cu).
#define LCR_THROW(status, ...)                                  \
  do {                                                          \
    char _b[512];                                               \
    snprintf(_b, sizeof _b, __VA_ARGS__);                       \
    throw LcrError{status, std::string(_b)};                    \
  } while (0)

#define CUDA_TRY(expr)                                                                      \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      lcr_status _s = _e == cudaErrorMemoryAllocation ? LCR_ERR_OOM : LCR_ERR_CUDA;         \
      LCR_THROW(_s, "%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e));     \
    }                                                                                       \
  } while (0)

// Every kernel launch goes through LCR_LAUNCH so that the context counts it and
// launch errors surface immediately.
#define LCR_LAUNCH(ctx, kernel, grid, block, smem, ...)                        \
  do {                                                                         \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);           \
    (ctx)->launches++;                                                         \
    CUDA_TRY(cudaGetLastError());                                              \
  } while (0)

// ---------------------------------------------------------- search index
// Morton-sorted points grouped into leaves of 32 (one warp-wide float4 load per
// leaf) with a 32-ary hierarchy of axis-aligned boxes above them.
constexpr int kMaxLevels = 6;  // root level <= 5: up to 32^6 = 2^30 points per cloud

struct IndexView {
  const float4* pts;            // npad = nleaf*32 sorted points, w = original index (int bits), sentinel NaN / -1
  const float4* lo[kMaxLevels]; // boxes per level; level 0 = leaves
  const float4* hi[kMaxLevels];
  int count[kMaxLevels];        // boxes per level
  int top;                      // level of the root (count[top] == 1)
  int n;                        // points (including non-finite ones, which become sentinels)
  int nleaf;
};

struct Index {
  IndexView v;
  void* block = nullptr;        // one allocation holding everything
  size_t bytes = 0;
  int refs = 1;                 // clouds with identical points in the same order share one index
};

// ------------------------------------------------------------------ cloud
// The exact k nearest neighbours (unordered (distance, index) keys, index in
// the numbering of the cloud they were searched in) that StatisticalOutlier-
// Removal found for every input point, handed to its inlier cloud: the k'
// nearest inliers of an inlier are the first k' inliers of its list whenever
// the list holds at least k' of them, so NormalEstimation on the inliers can
// select instead of searching again (the first normals call on the cloud
// consumes and releases them).  One allocation: keys, then keep flags, rank
// (input index -> inlier index), kept (inlier index -> input index).
struct NbrHint {
  void* block = nullptr;
  const unsigned long long* keys;  // [n_src][K]
  const uint8_t* keep;             // [n_src]
  const uint32_t* rank;            // [n_src], valid where keep
  const uint32_t* kept;            // [n_kept]
  int K = 0;
  int n_src = 0;
};

// The exact k nearest neighbours NormalEstimation found for every point of its
// output cloud (LCR_NORMALS_KEEP_NEIGHBOURS, k <= kGraphMaxK).  Row i (32
// words, 128 B) holds in words [0, k) the original indices of point i's k
// nearest, itself included, in no particular order, and in word kGraphR the
// largest squared distance among them as float bits (+inf when the cloud has
// fewer than k finite points, so that the row lists all of them).  Rows of
// non-finite points are not written: such a point is never a neighbour or a
// correspondence.  ICP against the cloud proves most correspondences from
// these rows instead of searching (icp.cu, k_icp_search).
constexpr int kGraphMaxK = 31;
constexpr int kGraphR = 31;
struct NbrGraph {
  uint32_t* rows = nullptr;     // [n][32]
  int k = 0;
};

struct lcr_cloud {
  size_t n = 0;
  float4* xyz = nullptr;        // x y z 0
  float4* nrm = nullptr;        // nx ny nz curvature
  uint32_t* rgb = nullptr;      // packed b g r a (little-endian PCL rgba)
  Index* index = nullptr;       // built on first search, freed with the cloud
  NbrHint* nbr = nullptr;       // SOR inliers only: their source's neighbour lists
  NbrGraph* graph = nullptr;    // normals output with LCR_NORMALS_KEEP_NEIGHBOURS only
};

struct lcr_ctx {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  uint64_t launches = 0;
  std::string last_error;
  // pinned host staging for small results
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  // persistent ICP device buffers (state + partial sums)
  void* icp_block = nullptr;
  size_t icp_bytes = 0;
  // captured ICP loops (one per method), reused across calls
  cudaGraphExec_t icp_exec[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};  // [method][solve width]
  int icp_graph_ok = -1;        // -1 unknown, 0 unavailable, 1 usable
  // optional event timing of selected kernels (lcr_kernel_timing)
  bool timing = false;
  struct KTimer {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    double ms = 0.0;
    uint64_t launches = 0;
  } kt[LCR_KT_COUNT];
  std::vector<cudaEvent_t> event_pool;
  // launch shapes (lcr_tune_set / lcr_autotune); the defaults are the hand-tuned ones
  struct Tune {
    int sor_warps = 5;      // warps per block of k_sor_dist
    int ne_warps = 5;       // warps per block of k_normals, k_normals_queued
    int icp_bps = 4;        // persistent blocks per SM of the batched ICP search kernels
  } tune;
};

// Brackets one launch with events when timing is on (see lcr_kernel_timing).
struct KernelTimer {
  lcr_ctx* ctx;
  int which;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelTimer(lcr_ctx* c, int w);
  ~KernelTimer();
};

// --------------------------------------------------------- memory helpers
void* dev_alloc(lcr_ctx* ctx, size_t bytes);
void dev_free(lcr_ctx* ctx, void* p);
void* pinned(lcr_ctx* ctx, size_t bytes);
lcr_cloud* cloud_alloc(lcr_ctx* ctx, size_t n);
void cloud_release(lcr_ctx* ctx, lcr_cloud* c);
const Index& cloud_index(lcr_ctx* ctx, const lcr_cloud* c);
void sync(lcr_ctx* ctx);

// --------------------------------------------------------- exact FP32 ops
// Squared distance exactly as FLANN's L2_Simple<float> evaluates it on three
// components: d = q - p, r = d0*d0; r += d1*d1; r += d2*d2 -- separate IEEE
// multiplies and adds (never contracted to FMA), so the GPU reproduces the CPU
// bit for bit.
__device__ __forceinline__ float exact_dist2(float qx, float qy, float qz, float px, float py, float pz) {
  const float d0 = __fsub_rn(qx, px), d1 = __fsub_rn(qy, py), d2 = __fsub_rn(qz, pz);
  return __fadd_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1)), __fmul_rn(d2, d2));
}

// Paired FP32 (sm_100 family): two IEEE single-precision operations in one
// instruction on a 64-bit register holding {low half, high half}, each half
// rounded to nearest like the scalar __fsub_rn / __fmul_rn.  A paired product
// feeding a paired add may still be fused into a paired FMA by the assembler
// (an exact_dist2 one ulp off was observed), so sums of products stay scalar
// __fadd_rn, which is never fused.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f32x2_dup(float a) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a));
  return r;
}
__device__ __forceinline__ float f32x2_lo(f32x2 v) { return __uint_as_float(static_cast<uint32_t>(v)); }
__device__ __forceinline__ float f32x2_hi(f32x2 v) { return __uint_as_float(static_cast<uint32_t>(v >> 32)); }
__device__ __forceinline__ f32x2 f32x2_sub(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 f32x2_mul(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// exact_dist2 of one query (each coordinate duplicated into both halves) to
// two points (x, y, z pairs): differences and squares paired, the two sums
// scalar; d0 and d1 are bit-identical to exact_dist2 of the low and high point.
__device__ __forceinline__ void exact_dist2_x2(f32x2 qx, f32x2 qy, f32x2 qz, f32x2 px, f32x2 py, f32x2 pz, float& d0,
                                               float& d1) {
  const f32x2 e0 = f32x2_sub(qx, px), e1 = f32x2_sub(qy, py), e2 = f32x2_sub(qz, pz);
  const f32x2 s0 = f32x2_mul(e0, e0), s1 = f32x2_mul(e1, e1), s2 = f32x2_mul(e2, e2);
  d0 = __fadd_rn(__fadd_rn(f32x2_lo(s0), f32x2_lo(s1)), f32x2_lo(s2));
  d1 = __fadd_rn(__fadd_rn(f32x2_hi(s0), f32x2_hi(s1)), f32x2_hi(s2));
}

// Lower bound of exact_dist2 over every point inside [lo, hi]: each per-axis gap
// is a rounded difference no larger than the corresponding point difference and
// rounding is monotone, so the bound never exceeds a member's distance.
__device__ __forceinline__ float box_dist2(const float4 lo, const float4 hi, float x, float y, float z) {
  const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, x), __fsub_rn(x, hi.x)), 0.f);
  const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, y), __fsub_rn(y, hi.y)), 0.f);
  const float gz = fmaxf(fmaxf(__fsub_rn(lo.z, z), __fsub_rn(z, hi.z)), 0.f);
  return __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
}

// Lower bound between any point of box a and any point of box b.
__device__ __forceinline__ float box_box_dist2(const float4 alo, const float4 ahi, const float4 blo, const float4 bhi) {
  const float gx = fmaxf(fmaxf(__fsub_rn(alo.x, bhi.x), __fsub_rn(blo.x, ahi.x)), 0.f);
  const float gy = fmaxf(fmaxf(__fsub_rn(alo.y, bhi.y), __fsub_rn(blo.y, ahi.y)), 0.f);
  const float gz = fmaxf(fmaxf(__fsub_rn(alo.z, bhi.z), __fsub_rn(blo.z, ahi.z)), 0.f);
  return __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
}

// (distance, index) packed so that integer order is (distance, then index) order.
__device__ __forceinline__ unsigned long long make_key(float d, uint32_t idx) {
  return (static_cast<unsigned long long>(__float_as_uint(d)) << 32) | idx;
}
__device__ __forceinline__ float key_dist(unsigned long long k) { return __uint_as_float(static_cast<uint32_t>(k >> 32)); }
__device__ __forceinline__ uint32_t key_idx(unsigned long long k) { return static_cast<uint32_t>(k); }

// 3x4 FP32 rigid transform applied as Eigen evaluates Matrix4f * Vector4f:
// ((r0*x + r1*y) + r2*z) + t with separate roundings.
struct Xf {
  float m[12];
};
__device__ __forceinline__ float3 xf_apply(const Xf& T, float x, float y, float z) {
  float3 o;
  o.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T.m[0], x), __fmul_rn(T.m[1], y)), __fmul_rn(T.m[2], z)), T.m[3]);
  o.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T.m[4], x), __fmul_rn(T.m[5], y)), __fmul_rn(T.m[6], z)), T.m[7]);
  o.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T.m[8], x), __fmul_rn(T.m[9], y)), __fmul_rn(T.m[10], z)), T.m[11]);
  return o;
}
__device__ __forceinline__ float3 xf_rotate(const Xf& T, float x, float y, float z) {
  float3 o;
  o.x = __fadd_rn(__fadd_rn(__fmul_rn(T.m[0], x), __fmul_rn(T.m[1], y)), __fmul_rn(T.m[2], z));
  o.y = __fadd_rn(__fadd_rn(__fmul_rn(T.m[4], x), __fmul_rn(T.m[5], y)), __fmul_rn(T.m[6], z));
  o.z = __fadd_rn(__fadd_rn(__fmul_rn(T.m[8], x), __fmul_rn(T.m[9], y)), __fmul_rn(T.m[10], z));
  return o;
}

__device__ __forceinline__ bool finite3(float x, float y, float z) {
  return isfinite(x) && isfinite(y) && isfinite(z);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(LCR_FULL, v, o);
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(LCR_FULL, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(LCR_FULL, v, o));
  return v;
}

// ---------------------------------------------------- shared primitives
// Stable LSD radix sort of (key, value) pairs on the context stream.  keys/vals
// are sorted in place (tmp buffers allocated internally).  `bits` = significant
// key bits (rounded up to 8-bit digits).
void radix_sort_pairs(lcr_ctx* ctx, uint32_t* keys, uint32_t* vals, int n, int bits);
// Order-preserving compaction: indices of flags[i] != 0 written to out_idx in
// ascending order.  Returns the count (synchronises).
int compact_flags(lcr_ctx* ctx, const uint8_t* flags, int n, uint32_t* out_idx);
void compact_flags_async(lcr_ctx* ctx, const uint8_t* flags, int n, uint32_t* out_idx, uint32_t* count_dev = nullptr);
// Gathers cloud rows: out[j] = in[idx[j]].
void gather_cloud(lcr_ctx* ctx, const lcr_cloud* in, const uint32_t* idx, int n, lcr_cloud* out);
// RMS over each cloud's finite points of |Ta p - Tb p| (synth.cu); host Ta, Tb [n][16], out [n].
void rmse_batch(lcr_ctx* ctx, const lcr_cloud* const* clouds, int n, const double* Ta, const double* Tb, double* out);
// Seeded synthetic capture pairs (synth.cu); allocates src[i], tgt[i].
void synth_depth(lcr_ctx* ctx, uint64_t seed, int npairs, const lcr_synth_params* prm, const lcr_render_params* cam,
                 const float* distance, const float* points, void* d_out, float* transforms);
void synth_turntable(lcr_ctx* ctx, uint64_t seed, int views, float step_deg, const lcr_render_params* cam,
                     float distance, int noise, void* d_out, float* poses);
void synth_pairs(lcr_ctx* ctx, uint64_t seed, int npairs, int npts, const lcr_synth_params* prm, lcr_cloud** src,
                 lcr_cloud** tgt, float* transforms);
// Device-side bounding box of the finite points of an xyz array: out[0] = lo, out[1] = hi.
void bbox(lcr_ctx* ctx, const float4* xyz, int n, float4* out2);

// ------------------------------------------------------------ index build
Index* build_index(lcr_ctx* ctx, const float4* xyz, int n);
Index* subset_index(lcr_ctx* ctx, const Index& src, const uint8_t* keep, const uint32_t* kept, int nkeep);
Index* share_index(Index* ix);
void free_index(lcr_ctx* ctx, Index* ix);

// ----------------------------------------------------- algorithm entry points
void knn_run(lcr_ctx* ctx, const lcr_cloud* ref, const lcr_cloud* query, int k, float cap, int32_t* d_idx,
             float* d_dist);
int backproject_run(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p, lcr_cloud** out);
void burst_fuse_run(lcr_ctx* ctx, const void* d_frames, const lcr_depth_params* p, void* d_out);
void backproject_into_run(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p, lcr_point* d_points,
                          size_t capacity, uint32_t* d_count);
lcr_cloud* voxel_run(lcr_ctx* ctx, const lcr_cloud* in, float lx, float ly, float lz);
void sor_run(lcr_ctx* ctx, const lcr_cloud* in, int mean_k, double std_mul, lcr_cloud** inliers,
             lcr_cloud** outliers, lcr_sor_stats* stats, float* host_dist);
lcr_cloud* normals_run(lcr_ctx* ctx, const lcr_cloud* in, int k, const float vp[3], int flags);
// SfM-side filters (sfm.cu).
void crop_box_run(lcr_ctx* ctx, const lcr_cloud* in, const float lo[3], const float hi[3], lcr_cloud** inside,
                  lcr_cloud** outside);
void euclidean_clusters_run(lcr_ctx* ctx, const lcr_cloud* in, double tolerance, size_t min_size, size_t max_size,
                            int32_t* host_labels, size_t* nclusters, lcr_cloud** clustered, lcr_cloud** rest);
void plane_segment_run(lcr_ctx* ctx, const lcr_cloud* in, double threshold, int hypotheses, uint64_t seed,
                       float coefficients[4], size_t* ninliers, lcr_cloud** plane, lcr_cloud** rest);
// Super-resolution front end (sr.cu).
// frames and out are uint16 (Kinect v1) or, with f32, float (Kinect v2).
void super_resolve_run(lcr_ctx* ctx, const void* frames, bool f32, int w, int h, int F, int factor, int max_iter,
                       double eps, void* out, float* warps_out, float minmax_out[2], int* iters_out);
// Launch-shape tuning (tune.cu).
void tune_apply(lcr_ctx* ctx, const lcr_tune& t);
lcr_tune tune_current(const lcr_ctx* ctx);
void autotune_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const char* cache_path,
                  lcr_tune_report* rep);
// Drops the captured ICP loops (their launch shapes changed).
void icp_graphs_reset(lcr_ctx* ctx);
// Takes the accumulated event time of a timed kernel (ms) and clears it.
double kernel_time_take(lcr_ctx* ctx, int which);
void icp_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const lcr_icp_params* p, const float* guess,
             lcr_icp_result* res);
void icp_batch_run(lcr_ctx* ctx, const lcr_cloud* const* src, const lcr_cloud* const* tgt, int npairs,
                   const lcr_icp_params* p, const float* guesses, lcr_icp_result* res);
void corr_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const double* T, double dmax, int32_t* d_idx,
              float* d_dist);
void crop_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double radius, uint8_t* d_removed);
lcr_cloud* transform_run(lcr_ctx* ctx, const lcr_cloud* in, const float* m);
// c4 = {x, y, z, finite count}, FP64 accumulation (synchronises).
void centroid_run(lcr_ctx* ctx, const lcr_cloud* in, double* c4);
// Same on the device, no synchronisation: out4 (device, 4 doubles) and, if
// outf is not null, the mean as 3 floats (device).
void centroid_device(lcr_ctx* ctx, const lcr_cloud* in, double* out4, float* outf);
lcr_cloud* upload_records(lcr_ctx* ctx, const void* recs, size_t n, bool device_src);
lcr_cloud* upload_xyz(lcr_ctx* ctx, const float* xyz, size_t n);
void download_records(lcr_ctx* ctx, const lcr_cloud* c, void* out);
lcr_cloud* concat_clouds(lcr_ctx* ctx, const lcr_cloud* a, const lcr_cloud* b);
// Largest float whose double value is <= v (PCL compares a float distance with a
// double squared threshold).
float float_cap(double v);

#define LCR_INF_HOST __builtin_huge_valf()
