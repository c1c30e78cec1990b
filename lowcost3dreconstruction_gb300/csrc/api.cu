// The C ABI (include/lcr.h).  Every entry point validates its arguments,
// selects the context's device, runs on the context stream and converts
// internal errors into an lcr_status plus a message (lcr_last_error).
#include <cmath>
#include <cstring>
#include <new>

#include "lcr_internal.cuh"
#include "posenet.cuh"

namespace {

#define API_BEGIN(ctx)                                \
  if (!(ctx)) return LCR_ERR_INVALID_ARG;             \
  try {                                               \
    CUDA_TRY(cudaSetDevice((ctx)->device));

#define API_END(ctx)                                                   \
  }                                                                    \
  catch (const LcrError& e) {                                          \
    (ctx)->last_error = e.msg;                                         \
    return e.st;                                                       \
  }                                                                    \
  catch (const std::bad_alloc&) {                                      \
    (ctx)->last_error = "host allocation failed";                      \
    return LCR_ERR_OOM;                                                \
  }                                                                    \
  catch (...) {                                                        \
    (ctx)->last_error = "unknown error";                               \
    return LCR_ERR_CUDA;                                               \
  }

#define REQUIRE(cond, ...)                                  \
  do {                                                      \
    if (!(cond)) LCR_THROW(LCR_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

__global__ void k_finite_flags(const float4* __restrict__ xyz, size_t n, uint8_t* __restrict__ out) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) {
    const float4 p = xyz[i];
    out[i] = finite3(p.x, p.y, p.z) ? 1 : 0;
  }
}

__global__ void k_invert(const uint8_t* __restrict__ in, size_t n, uint8_t* __restrict__ out) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[i] ? 0 : 1;
}

void check_depth(const lcr_depth_params* p) {
  REQUIRE(p, "null depth parameters");
  REQUIRE(p->model == LCR_DEPTH_KINECT_V1 || p->model == LCR_DEPTH_KINECT_V2 || p->model == LCR_DEPTH_PINHOLE_F32,
          "unknown depth model %d", p->model);
  REQUIRE(p->width > 0 && p->height > 0 && static_cast<long long>(p->width) * p->height < (1LL << 31),
          "bad image size %dx%d", p->width, p->height);
  REQUIRE(p->frames >= 1 && p->frames <= 4096, "frames must be in [1, 4096]");
  REQUIRE(p->fx != 0 && p->fy != 0, "zero focal length");
}

size_t depth_bytes(const lcr_depth_params* p) {
  return static_cast<size_t>(p->width) * p->height * p->frames * (p->model == LCR_DEPTH_KINECT_V1 ? 2 : 4);
}

}  // namespace

extern "C" {

const char* lcr_status_string(lcr_status s) {
  switch (s) {
    case LCR_OK: return "ok";
    case LCR_ERR_INVALID_ARG: return "invalid argument";
    case LCR_ERR_EMPTY: return "empty cloud";
    case LCR_ERR_NO_CORRESPONDENCES: return "not enough correspondences";
    case LCR_NOT_CONVERGED: return "not converged";
    case LCR_ERR_CUDA: return "CUDA error";
    case LCR_ERR_TIMEOUT: return "device wait timed out";
    case LCR_ERR_OOM: return "out of memory";
    case LCR_ERR_IO: return "I/O error";
    case LCR_ERR_TOO_FEW_POINTS: return "too few points for k neighbours";
    case LCR_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

lcr_status lcr_ctx_create(lcr_ctx** out, int device) {
  if (!out) return LCR_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return LCR_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return LCR_ERR_INVALID_ARG;
  lcr_ctx* ctx = new (std::nothrow) lcr_ctx();
  if (!ctx) return LCR_ERR_OOM;
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return LCR_ERR_CUDA;
  }
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
  *out = ctx;
  return LCR_OK;
}

void lcr_ctx_destroy(lcr_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& per_method : ctx->icp_exec)
    for (cudaGraphExec_t e : per_method)
      if (e) cudaGraphExecDestroy(e);
  for (auto& t : ctx->kt)
    for (auto& e : t.pending) {
      cudaEventDestroy(e.first);
      cudaEventDestroy(e.second);
    }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->icp_block) cudaFree(ctx->icp_block);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  cudaStreamDestroy(ctx->stream);
  cudaGetLastError();
  delete ctx;
}

const char* lcr_last_error(const lcr_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

lcr_status lcr_ctx_synchronize(lcr_ctx* ctx) {
  API_BEGIN(ctx)
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

void* lcr_ctx_stream(lcr_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

uint64_t lcr_ctx_launch_count(const lcr_ctx* ctx) { return ctx ? ctx->launches : 0; }

lcr_status lcr_kernel_timing(lcr_ctx* ctx, int enable) {
  API_BEGIN(ctx)
  sync(ctx);
  for (auto& t : ctx->kt) {
    for (auto& e : t.pending) {
      ctx->event_pool.push_back(e.first);
      ctx->event_pool.push_back(e.second);
    }
    t.pending.clear();
    t.ms = 0.0;
    t.launches = 0;
  }
  ctx->timing = enable != 0;
  return LCR_OK;
  API_END(ctx)
}

lcr_status lcr_kernel_time(lcr_ctx* ctx, int which, double* ms, uint64_t* launches) {
  API_BEGIN(ctx)
  REQUIRE(which >= 0 && which < LCR_KT_COUNT, "unknown timed kernel %d", which);
  sync(ctx);
  auto& t = ctx->kt[which];
  for (auto& e : t.pending) {
    float v = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&v, e.first, e.second));
    t.ms += v;
    t.launches += 1;
    ctx->event_pool.push_back(e.first);
    ctx->event_pool.push_back(e.second);
  }
  t.pending.clear();
  if (ms) *ms = t.ms;
  if (launches) *launches = t.launches;
  return LCR_OK;
  API_END(ctx)
}

// ------------------------------------------------------------------ clouds
lcr_status lcr_cloud_upload(lcr_ctx* ctx, const lcr_point* pts, size_t n, lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(out && (pts || n == 0), "null argument");
  REQUIRE(n < (1u << 31), "cloud too large");
  *out = upload_records(ctx, pts, n, false);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_cloud_upload_xyz(lcr_ctx* ctx, const float* xyz, size_t n, lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(out && (xyz || n == 0), "null argument");
  REQUIRE(n < (1u << 31), "cloud too large");
  *out = upload_xyz(ctx, xyz, n);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_cloud_from_device(lcr_ctx* ctx, const void* d_pts, size_t n, lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(out && (d_pts || n == 0), "null argument");
  REQUIRE(n < (1u << 31), "cloud too large");
  *out = upload_records(ctx, d_pts, n, true);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

size_t lcr_cloud_size(const lcr_cloud* c) { return c ? c->n : 0; }

lcr_status lcr_cloud_download(lcr_ctx* ctx, const lcr_cloud* c, lcr_point* out, size_t capacity) {
  API_BEGIN(ctx)
  REQUIRE(c && (out || c->n == 0), "null argument");
  REQUIRE(capacity >= c->n, "capacity %zu < cloud size %zu", capacity, c->n);
  download_records(ctx, c, out);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_cloud_neighbours(lcr_ctx* ctx, const lcr_cloud* c, int* k, uint32_t* host_rows) {
  API_BEGIN(ctx)
  REQUIRE(c && k, "null argument");
  *k = c->graph ? c->graph->k : 0;
  REQUIRE(c->graph, "the cloud holds no neighbour rows (lcr_normals with LCR_NORMALS_KEEP_NEIGHBOURS makes them)");
  if (host_rows && c->n) {
    CUDA_TRY(cudaMemcpyAsync(host_rows, c->graph->rows, sizeof(uint32_t) * 32 * c->n, cudaMemcpyDeviceToHost,
                             ctx->stream));
    sync(ctx);
  }
  API_END(ctx)
  return LCR_OK;
}

void lcr_cloud_free(lcr_ctx* ctx, lcr_cloud* c) {
  if (!ctx || !c) return;
  try {
    cudaSetDevice(ctx->device);
    cloud_release(ctx, c);
  } catch (...) {
  }
}

lcr_status lcr_cloud_concat(lcr_ctx* ctx, const lcr_cloud* a, const lcr_cloud* b, lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(a && b && out, "null argument");
  *out = concat_clouds(ctx, a, b);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

// --------------------------------------------------------- back-projection
lcr_status lcr_backproject_device(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p, lcr_cloud** out) {
  API_BEGIN(ctx)
  check_depth(p);
  REQUIRE(d_depth && out, "null argument");
  backproject_run(ctx, d_depth, p, out);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_backproject_into(lcr_ctx* ctx, const void* d_depth, const lcr_depth_params* p, lcr_point* d_points,
                                size_t capacity, uint32_t* d_count) {
  API_BEGIN(ctx)
  check_depth(p);
  REQUIRE(d_depth && d_count && (d_points || capacity == 0), "null argument");
  // the records are stored as two 16-byte vectors each, the count as one word
  REQUIRE(reinterpret_cast<uintptr_t>(d_points) % 16 == 0 && reinterpret_cast<uintptr_t>(d_count) % 4 == 0,
          "d_points must be 16-byte aligned and d_count 4-byte aligned");
  backproject_into_run(ctx, d_depth, p, d_points, capacity, d_count);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_backproject(lcr_ctx* ctx, const void* depth, const lcr_depth_params* p, lcr_cloud** out) {
  API_BEGIN(ctx)
  check_depth(p);
  REQUIRE(depth && out, "null argument");
  const size_t bytes = depth_bytes(p);
  void* d = dev_alloc(ctx, bytes);
  CUDA_TRY(cudaMemcpyAsync(d, depth, bytes, cudaMemcpyHostToDevice, ctx->stream));
  backproject_run(ctx, d, p, out);
  dev_free(ctx, d);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_burst_fuse(lcr_ctx* ctx, const void* frames, const lcr_depth_params* p, void* fused_out) {
  API_BEGIN(ctx)
  check_depth(p);
  REQUIRE(frames && fused_out, "null argument");
  const size_t bytes = depth_bytes(p);
  const size_t obytes = bytes / p->frames;
  char* d = static_cast<char*>(dev_alloc(ctx, bytes + obytes));
  CUDA_TRY(cudaMemcpyAsync(d, frames, bytes, cudaMemcpyHostToDevice, ctx->stream));
  burst_fuse_run(ctx, d, p, d + bytes);
  CUDA_TRY(cudaMemcpyAsync(fused_out, d + bytes, obytes, cudaMemcpyDeviceToHost, ctx->stream));
  dev_free(ctx, d);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

// ----------------------------------------------------------------- filters
lcr_status lcr_voxel_grid(lcr_ctx* ctx, const lcr_cloud* in, float lx, float ly, float lz, lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(in && out, "null argument");
  *out = voxel_run(ctx, in, lx, ly, lz);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_sor(lcr_ctx* ctx, const lcr_cloud* in, int mean_k, double std_mul, lcr_cloud** inliers,
                   lcr_cloud** outliers, lcr_sor_stats* stats) {
  API_BEGIN(ctx)
  REQUIRE(in, "null argument");
  if (inliers) *inliers = nullptr;
  if (outliers) *outliers = nullptr;
  sor_run(ctx, in, mean_k, std_mul, inliers, outliers, stats, nullptr);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_sor_distances(lcr_ctx* ctx, const lcr_cloud* in, int mean_k, float* distances, lcr_sor_stats* stats) {
  API_BEGIN(ctx)
  REQUIRE(in && distances, "null argument");
  lcr_sor_stats local;
  sor_run(ctx, in, mean_k, 1.0, nullptr, nullptr, stats ? stats : &local, distances);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_normals(lcr_ctx* ctx, const lcr_cloud* in, int k, const float viewpoint[3], int flags,
                       lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(in && out, "null argument");
  const float zero[3] = {0.f, 0.f, 0.f};
  *out = normals_run(ctx, in, k, viewpoint ? viewpoint : zero, flags);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

// --------------------------------------------------------------------- ICP
void lcr_icp_params_default(lcr_icp_params* p) {
  if (!p) return;
  p->max_correspondence_distance = 0.1;
  p->max_iterations = 50;
  p->transformation_epsilon = 1e-9;
  p->euclidean_fitness_epsilon = 0.001;
  p->method = LCR_ICP_POINT_TO_POINT;
  p->compute_fitness = 1;
  p->stop_iteration = 0;
  p->stop_rms = 0.0;
}

lcr_status lcr_icp(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const lcr_icp_params* p,
                   const float guess[16], lcr_icp_result* res, lcr_cloud** registered) {
  lcr_status st = LCR_OK;
  API_BEGIN(ctx)
  REQUIRE(src && tgt && p && res, "null argument");
  REQUIRE(p->method == LCR_ICP_POINT_TO_POINT || p->method == LCR_ICP_POINT_TO_PLANE, "unknown ICP method");
  REQUIRE(p->stop_iteration >= 0 && p->stop_rms >= 0, "negative stop rule");
  if (registered) *registered = nullptr;
  icp_run(ctx, src, tgt, p, guess, res);
  if (registered) *registered = transform_run(ctx, src, res->transform);
  sync(ctx);
  if (res->state == LCR_ICP_STATE_NO_CORRESPONDENCES) {
    ctx->last_error = "not enough correspondences found";
    st = LCR_ERR_NO_CORRESPONDENCES;
  }
  API_END(ctx)
  return st;
}

lcr_status lcr_icp_batch(lcr_ctx* ctx, const lcr_cloud* const* src, const lcr_cloud* const* tgt, size_t npairs,
                         const lcr_icp_params* p, const float* guesses, lcr_icp_result* results) {
  lcr_status st = LCR_OK;
  API_BEGIN(ctx)
  REQUIRE(p && (npairs == 0 || (src && tgt && results)), "null argument");
  REQUIRE(npairs < (1u << 20), "too many pairs (%zu)", npairs);
  REQUIRE(p->method == LCR_ICP_POINT_TO_POINT || p->method == LCR_ICP_POINT_TO_PLANE, "unknown ICP method");
  REQUIRE(p->stop_iteration >= 0 && p->stop_rms >= 0, "negative stop rule");
  icp_batch_run(ctx, src, tgt, static_cast<int>(npairs), p, guesses, results);
  for (size_t i = 0; i < npairs; ++i)
    if (results[i].state == LCR_ICP_STATE_NO_CORRESPONDENCES) {
      ctx->last_error = "not enough correspondences found (pair " + std::to_string(i) + ")";
      st = LCR_ERR_NO_CORRESPONDENCES;
      break;
    }
  API_END(ctx)
  return st;
}

lcr_status lcr_correspondences(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const double T[16],
                               double max_correspondence_distance, int32_t* idx, float* dist) {
  API_BEGIN(ctx)
  REQUIRE(src && tgt && T && idx && dist, "null argument");
  const size_t n = src->n;
  if (n) {
    char* d = static_cast<char*>(dev_alloc(ctx, n * 8));
    corr_run(ctx, src, tgt, T, max_correspondence_distance, reinterpret_cast<int32_t*>(d),
             reinterpret_cast<float*>(d + n * 4));
    CUDA_TRY(cudaMemcpyAsync(idx, d, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(dist, d + n * 4, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    dev_free(ctx, d);
  }
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_knn(lcr_ctx* ctx, const lcr_cloud* ref, const lcr_cloud* query, int k, float max_dist_sq,
                   int32_t* idx, float* dist) {
  API_BEGIN(ctx)
  REQUIRE(ref && query && idx && dist, "null argument");
  REQUIRE(k >= 1 && k <= 512, "k must be in [1, 512]");
  const size_t m = query->n * static_cast<size_t>(k);
  if (m) {
    char* d = static_cast<char*>(dev_alloc(ctx, m * 8));
    const float cap = max_dist_sq < 0 ? LCR_INF_HOST : max_dist_sq;
    knn_run(ctx, ref, query, k, cap, reinterpret_cast<int32_t*>(d), reinterpret_cast<float*>(d + m * 4));
    CUDA_TRY(cudaMemcpyAsync(idx, d, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(dist, d + m * 4, m * 4, cudaMemcpyDeviceToHost, ctx->stream));
    dev_free(ctx, d);
  }
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

// -------------------------------------------------------------- accumulate
lcr_status lcr_crop_redundant(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double radius,
                              uint8_t* removed) {
  API_BEGIN(ctx)
  REQUIRE(src && tgt && (removed || src->n == 0), "null argument");
  REQUIRE(radius >= 0, "negative radius");
  if (src->n) {
    uint8_t* d = static_cast<uint8_t*>(dev_alloc(ctx, src->n));
    crop_run(ctx, src, tgt, radius, d);
    CUDA_TRY(cudaMemcpyAsync(removed, d, src->n, cudaMemcpyDeviceToHost, ctx->stream));
    dev_free(ctx, d);
  }
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_accumulate(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double radius, int k,
                          double std_mul, int flags, lcr_cloud** out, lcr_cloud** remaining) {
  API_BEGIN(ctx)
  REQUIRE(src && tgt && out, "null argument");
  REQUIRE(radius >= 0 && k > 0, "bad radius or k");
  lcr_cloud empty;
  lcr_cloud* rem = nullptr;
  if (flags & LCR_ACCUM_ALL) {
    rem = concat_clouds(ctx, src, &empty);
  } else {
    const size_t n = src->n;
    uint8_t* removed = static_cast<uint8_t*>(dev_alloc(ctx, 2 * n + 16));
    uint8_t* keep = removed + n;
    uint32_t* idx = static_cast<uint32_t*>(dev_alloc(ctx, 4 * n + 16));
    crop_run(ctx, src, tgt, radius, removed);
    int nk = 0;
    if (n) {
      LCR_LAUNCH(ctx, k_invert, static_cast<unsigned>((n + 255) / 256), 256, 0, removed, n, keep);
      nk = compact_flags(ctx, keep, static_cast<int>(n), idx);
    }
    lcr_cloud* rem0 = cloud_alloc(ctx, nk);
    gather_cloud(ctx, src, idx, nk, rem0);
    dev_free(ctx, removed);
    dev_free(ctx, idx);
    // The reference's SOR reads past its results with <= k points; the cleaning
    // pass is skipped for such small remainders.
    if (nk > k) {
      lcr_cloud* inl = nullptr;
      sor_run(ctx, rem0, k, std_mul, &inl, nullptr, nullptr, nullptr);
      cloud_release(ctx, rem0);
      rem = inl;
    } else {
      rem = rem0;
    }
  }
  *out = concat_clouds(ctx, tgt, rem);
  if (remaining) *remaining = rem;
  else cloud_release(ctx, rem);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

// --------------------------------------------------- transforms, centroid
lcr_status lcr_transform(lcr_ctx* ctx, const lcr_cloud* in, const float m[16], lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(in && m && out, "null argument");
  *out = transform_run(ctx, in, m);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_centroid(lcr_ctx* ctx, const lcr_cloud* in, float centroid[4]) {
  API_BEGIN(ctx)
  REQUIRE(in && centroid, "null argument");
  double c4[4];
  centroid_run(ctx, in, c4);
  if (c4[3] == 0) LCR_THROW(LCR_ERR_EMPTY, "centroid of a cloud without finite points");
  for (int i = 0; i < 3; ++i) centroid[i] = static_cast<float>(c4[i]);
  centroid[3] = 1.f;
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_centroid_align(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double roll, double pitch,
                              double yaw, double elevation, lcr_cloud** out, float transform[16]) {
  API_BEGIN(ctx)
  REQUIRE(src && tgt && out, "null argument");
  double cs[4], ct[4];
  centroid_run(ctx, src, cs);
  centroid_run(ctx, tgt, ct);
  if (cs[3] == 0 || ct[3] == 0) LCR_THROW(LCR_ERR_EMPTY, "centroid_align needs non-empty clouds");
  const double d2r = 3.14159265358979323846 / 180.0;
  const double a = roll * d2r, b = pitch * d2r, c = yaw * d2r;
  const double Rx[9] = {1, 0, 0, 0, std::cos(a), -std::sin(a), 0, std::sin(a), std::cos(a)};
  const double Ry[9] = {std::cos(b), 0, std::sin(b), 0, 1, 0, -std::sin(b), 0, std::cos(b)};
  const double Rz[9] = {std::cos(c), -std::sin(c), 0, std::sin(c), std::cos(c), 0, 0, 0, 1};
  double Rxy[9], R[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      Rxy[3 * i + j] = Rx[3 * i] * Ry[j] + Rx[3 * i + 1] * Ry[3 + j] + Rx[3 * i + 2] * Ry[6 + j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = Rxy[3 * i] * Rz[j] + Rxy[3 * i + 1] * Rz[3 + j] + Rxy[3 * i + 2] * Rz[6 + j];
  // p' = R (p - c_s) + c_t + (0, e, 0)
  float m[16];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) m[4 * i + j] = static_cast<float>(R[3 * i + j]);
    const double t = ct[i] + (i == 1 ? elevation : 0.0) - (R[3 * i] * cs[0] + R[3 * i + 1] * cs[1] + R[3 * i + 2] * cs[2]);
    m[4 * i + 3] = static_cast<float>(t);
  }
  m[12] = m[13] = m[14] = 0.f;
  m[15] = 1.f;
  *out = transform_run(ctx, src, m);
  if (transform) std::memcpy(transform, m, sizeof(m));
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

}  // extern "C"

// ------------------------------------------------------------ pose proposal
namespace {

std::vector<posenet::CloudRef> cloud_refs(const lcr_cloud* const* a, const lcr_cloud* const* b, size_t n) {
  std::vector<posenet::CloudRef> r;
  r.reserve(b ? 2 * n : n);
  for (size_t i = 0; i < n; ++i) {
    if (!a[i]) LCR_THROW(LCR_ERR_INVALID_ARG, "null cloud %zu", i);
    r.push_back({a[i]->xyz, static_cast<long long>(a[i]->n)});
  }
  if (b)
    for (size_t i = 0; i < n; ++i) {
      if (!b[i]) LCR_THROW(LCR_ERR_INVALID_ARG, "null target cloud %zu", i);
      r.push_back({b[i]->xyz, static_cast<long long>(b[i]->n)});
    }
  return r;
}

void h2d(lcr_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (bytes) CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
}

void d2h(lcr_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (dst && bytes) CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
}

constexpr size_t kMaxPairs = 1u << 16;

}  // namespace

extern "C" {

lcr_status lcr_remove_nan(lcr_ctx* ctx, const lcr_cloud* in, lcr_cloud** out) {
  API_BEGIN(ctx)
  REQUIRE(in && out, "null argument");
  *out = nullptr;
  const size_t n = in->n;
  uint8_t* keep = static_cast<uint8_t*>(dev_alloc(ctx, n + 16));
  uint32_t* idx = static_cast<uint32_t*>(dev_alloc(ctx, 4 * n + 16));
  int nk = 0;
  if (n) {
    LCR_LAUNCH(ctx, k_finite_flags, static_cast<unsigned>((n + 255) / 256), 256, 0, in->xyz, n, keep);
    nk = compact_flags(ctx, keep, static_cast<int>(n), idx);
  }
  lcr_cloud* o = cloud_alloc(ctx, nk);
  gather_cloud(ctx, in, idx, nk, o);
  dev_free(ctx, keep);
  dev_free(ctx, idx);
  sync(ctx);
  *out = o;
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_crop_box(lcr_ctx* ctx, const lcr_cloud* in, const float min[3], const float max[3],
                        lcr_cloud** inside, lcr_cloud** outside) {
  API_BEGIN(ctx)
  REQUIRE(in && min && max, "null argument");
  if (inside) *inside = nullptr;
  if (outside) *outside = nullptr;
  crop_box_run(ctx, in, min, max, inside, outside);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_euclidean_clusters(lcr_ctx* ctx, const lcr_cloud* in, double tolerance, size_t min_size,
                                  size_t max_size, int32_t* labels, size_t* nclusters, lcr_cloud** clustered,
                                  lcr_cloud** rest) {
  API_BEGIN(ctx)
  REQUIRE(in && nclusters, "null argument");
  REQUIRE(tolerance > 0 && std::isfinite(tolerance), "tolerance must be positive");
  REQUIRE(in->n < (1u << 31), "cloud too large");
  if (clustered) *clustered = nullptr;
  if (rest) *rest = nullptr;
  euclidean_clusters_run(ctx, in, tolerance, min_size, max_size, labels, nclusters, clustered, rest);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_plane_segment(lcr_ctx* ctx, const lcr_cloud* in, double threshold, int hypotheses, uint64_t seed,
                             float coefficients[4], size_t* ninliers, lcr_cloud** plane, lcr_cloud** rest) {
  API_BEGIN(ctx)
  REQUIRE(in && coefficients && ninliers, "null argument");
  REQUIRE(threshold > 0 && std::isfinite(threshold), "threshold must be positive");
  REQUIRE(hypotheses >= 1 && hypotheses <= (1 << 20), "hypotheses must be in [1, 2^20]");
  REQUIRE(in->n < (1u << 31), "cloud too large");
  if (plane) *plane = nullptr;
  if (rest) *rest = nullptr;
  plane_segment_run(ctx, in, threshold, hypotheses, seed, coefficients, ninliers, plane, rest);
  API_END(ctx)
  return LCR_OK;
}

namespace {
void check_sr(const lcr_sr_params* p) {
  REQUIRE(p->width >= 1 && p->height >= 1 && static_cast<long long>(p->width) * p->height <= (1LL << 26),
          "bad image size %dx%d", p->width, p->height);
  REQUIRE(p->frames >= 1 && p->frames <= 1024, "frames must be in [1, 1024]");
  REQUIRE(p->factor >= 1 && p->factor <= 16, "factor must be in [1, 16]");
  REQUIRE(p->ecc_iterations >= 0 && p->ecc_epsilon >= 0, "bad ECC limits");
}
}  // namespace

lcr_status lcr_super_resolve(lcr_ctx* ctx, const uint16_t* frames, const lcr_sr_params* p, uint16_t* depth_out,
                             float* warps, float minmax[2], int32_t* iterations) {
  API_BEGIN(ctx)
  REQUIRE(p && frames && depth_out, "null argument");
  check_sr(p);
  super_resolve_run(ctx, frames, false, p->width, p->height, p->frames, p->factor, p->ecc_iterations,
                    p->ecc_epsilon, depth_out, warps, minmax, iterations);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_super_resolve_f32(lcr_ctx* ctx, const float* frames, const lcr_sr_params* p, float* depth_out,
                                 float* warps, float minmax[2], int32_t* iterations) {
  API_BEGIN(ctx)
  REQUIRE(p && frames && depth_out, "null argument");
  check_sr(p);
  super_resolve_run(ctx, frames, true, p->width, p->height, p->frames, p->factor, p->ecc_iterations, p->ecc_epsilon,
                    depth_out, warps, minmax, iterations);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_tune_get(lcr_ctx* ctx, lcr_tune* t) {
  API_BEGIN(ctx)
  REQUIRE(t, "null argument");
  *t = tune_current(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_tune_set(lcr_ctx* ctx, const lcr_tune* t) {
  API_BEGIN(ctx)
  REQUIRE(t, "null argument");
  sync(ctx);
  tune_apply(ctx, *t);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_autotune(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const char* cache_path,
                        lcr_tune_report* report) {
  API_BEGIN(ctx)
  REQUIRE(src && tgt && report, "null argument");
  REQUIRE(src->n > 64 && tgt->n > 0, "autotuning needs a source of more than 64 points and a target");
  autotune_run(ctx, src, tgt, cache_path, report);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_synthetic_pairs(lcr_ctx* ctx, uint64_t seed, size_t npairs, int points, const lcr_synth_params* p,
                               lcr_cloud** src, lcr_cloud** tgt, float* transforms) {
  API_BEGIN(ctx)
  REQUIRE(p && (npairs == 0 || (src && tgt && transforms)), "null argument");
  REQUIRE(npairs <= 65535, "too many pairs (%zu)", npairs);
  REQUIRE(points >= 1 && points <= (1 << 24), "points must be in [1, 2^24]");
  REQUIRE(p->yaw_deg >= 0.f && p->tilt_deg >= 0.f && p->translation >= 0.f, "ranges must be non-negative");
  for (size_t i = 0; i < npairs; ++i) src[i] = tgt[i] = nullptr;
  try {
    synth_pairs(ctx, seed, static_cast<int>(npairs), points, p, src, tgt, transforms);
  } catch (...) {
    for (size_t i = 0; i < npairs; ++i) {
      cloud_release(ctx, src[i]);
      cloud_release(ctx, tgt[i]);
      src[i] = tgt[i] = nullptr;
    }
    throw;
  }
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_synthetic_depth(lcr_ctx* ctx, uint64_t seed, size_t npairs, const lcr_synth_params* p,
                               const lcr_render_params* cam, const float* distance, const float* points,
                               void* d_depth, float* transforms) {
  API_BEGIN(ctx)
  REQUIRE(p && cam && (npairs == 0 || (d_depth && transforms)), "null argument");
  REQUIRE(npairs <= 32767, "too many pairs (%zu)", npairs);
  REQUIRE(cam->model == LCR_DEPTH_KINECT_V1 || cam->model == LCR_DEPTH_KINECT_V2 ||
              cam->model == LCR_DEPTH_PINHOLE_F32,
          "unknown depth model %d", cam->model);
  REQUIRE(cam->width >= 1 && cam->height >= 1 && static_cast<long long>(cam->width) * cam->height <= (1ll << 26),
          "image size %dx%d out of range", cam->width, cam->height);
  REQUIRE(cam->fx > 0 && cam->fy > 0 && std::isfinite(cam->cx) && std::isfinite(cam->cy), "bad intrinsics");
  REQUIRE(cam->samples_per_pixel >= 0 && cam->samples_per_pixel <= 64, "samples_per_pixel out of [0, 64]");
  REQUIRE(p->yaw_deg >= 0.f && p->tilt_deg >= 0.f && p->translation >= 0.f, "ranges must be non-negative");
  if (distance)
    for (size_t i = 0; i < npairs; ++i)
      REQUIRE(distance[i] >= 0.2f && distance[i] <= 20.f, "distance[%zu] out of [0.2, 20] m", i);
  REQUIRE(!(distance && points), "give distance or points, not both");
  if (points)
    for (size_t i = 0; i < npairs; ++i) REQUIRE(points[i] >= 1.f, "points[%zu] must be >= 1", i);
  synth_depth(ctx, seed, static_cast<int>(npairs), p, cam, distance, points, d_depth, transforms);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_synthetic_turntable(lcr_ctx* ctx, uint64_t seed, int views, float step_deg,
                                   const lcr_render_params* cam, float distance, int noise, void* d_depth,
                                   float* poses) {
  API_BEGIN(ctx)
  REQUIRE(cam && (views == 0 || (d_depth && poses)), "null argument");
  REQUIRE(views >= 0 && views <= 65535, "views out of [0, 65535]");
  REQUIRE(cam->model == LCR_DEPTH_KINECT_V1 || cam->model == LCR_DEPTH_KINECT_V2 ||
              cam->model == LCR_DEPTH_PINHOLE_F32,
          "unknown depth model %d", cam->model);
  REQUIRE(cam->width >= 1 && cam->height >= 1 && static_cast<long long>(cam->width) * cam->height <= (1ll << 26),
          "image size %dx%d out of range", cam->width, cam->height);
  REQUIRE(cam->fx > 0 && cam->fy > 0 && std::isfinite(cam->cx) && std::isfinite(cam->cy), "bad intrinsics");
  REQUIRE(cam->samples_per_pixel >= 0 && cam->samples_per_pixel <= 64, "samples_per_pixel out of [0, 64]");
  REQUIRE(distance >= 0.2f && distance <= 20.f && std::isfinite(step_deg), "distance out of [0.2, 20] m");
  synth_turntable(ctx, seed, views, step_deg, cam, distance, noise, d_depth, poses);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_rmse_batch(lcr_ctx* ctx, const lcr_cloud* const* clouds, size_t n, const double* Ta, const double* Tb,
                          double* out) {
  API_BEGIN(ctx)
  REQUIRE(n == 0 || (clouds && Ta && Tb && out), "null argument");
  REQUIRE(n <= (1u << 20), "too many clouds (%zu)", n);
  for (size_t i = 0; i < n; ++i) REQUIRE(clouds[i], "null cloud %zu", i);
  rmse_batch(ctx, clouds, static_cast<int>(n), Ta, Tb, out);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_create(lcr_ctx* ctx, uint64_t seed, lcr_posenet** net) {
  API_BEGIN(ctx)
  REQUIRE(net, "null argument");
  *net = nullptr;
  auto* n = new lcr_posenet();
  try {
    posenet::create(ctx, n, seed);
    sync(ctx);
  } catch (...) {
    if (n->block) dev_free(ctx, n->block);
    delete n;
    throw;
  }
  *net = n;
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_free(lcr_ctx* ctx, lcr_posenet* net) {
  API_BEGIN(ctx)
  if (net) {
    posenet::destroy(ctx, net);
    sync(ctx);
    delete net;
  }
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_get_params(lcr_ctx* ctx, const lcr_posenet* net, float* params) {
  API_BEGIN(ctx)
  REQUIRE(net && params, "null argument");
  d2h(ctx, params, net->w, posenet::kParams * sizeof(float));
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_set_params(lcr_ctx* ctx, lcr_posenet* net, const float* params) {
  API_BEGIN(ctx)
  REQUIRE(net && params, "null argument");
  h2d(ctx, net->w, params, posenet::kParams * sizeof(float));
  posenet::pack(ctx, net);
  sync(ctx);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_sample(lcr_ctx* ctx, const lcr_cloud* const* clouds, size_t n, uint64_t seed, float* pts,
                              double* centroids) {
  API_BEGIN(ctx)
  REQUIRE(n == 0 || clouds, "null argument");
  REQUIRE(n <= 2 * kMaxPairs, "too many clouds (%zu)", n);
  if (n) {
    const auto refs = cloud_refs(clouds, nullptr, n);
    char* d = static_cast<char*>(dev_alloc(ctx, n * (sizeof(posenet::CloudRef) + posenet::kPts * 16 + 24)));
    auto* dr = reinterpret_cast<posenet::CloudRef*>(d);
    auto* dp = reinterpret_cast<float4*>(d + n * sizeof(posenet::CloudRef));
    auto* dc = reinterpret_cast<double*>(d + n * (sizeof(posenet::CloudRef) + posenet::kPts * 16));
    h2d(ctx, dr, refs.data(), n * sizeof(posenet::CloudRef));
    posenet::sample(ctx, dr, static_cast<int>(n), seed, dp, dc);
    d2h(ctx, pts, dp, n * posenet::kPts * 16);
    d2h(ctx, centroids, dc, n * 24);
    sync(ctx);
    dev_free(ctx, d);
  }
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_forward(lcr_ctx* ctx, lcr_posenet* net, const float* pts, size_t npairs, int train,
                               float* features, int32_t* argmax, float* out) {
  API_BEGIN(ctx)
  REQUIRE(net && (npairs == 0 || pts), "null argument");
  REQUIRE(npairs <= kMaxPairs, "too many pairs (%zu)", npairs);
  if (npairs) {
    const auto b = posenet::batch(ctx, net, static_cast<int>(npairs), train != 0);
    h2d(ctx, b.pts, pts, 2 * npairs * posenet::kPts * 16);
    posenet::encode(ctx, net, b, train != 0);
    posenet::head_forward(ctx, net, b);
    d2h(ctx, features, b.feat, 2 * npairs * posenet::kF3 * 4);
    if (train) d2h(ctx, argmax, b.argmax, 2 * npairs * posenet::kF3 * 4);
    d2h(ctx, out, b.y, npairs * posenet::kOut * 4);
    posenet::check_error(ctx, net);
  }
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_gradients(lcr_ctx* ctx, lcr_posenet* net, const float* pts, const float* labels, size_t npairs,
                                 float* loss, float* grads) {
  API_BEGIN(ctx)
  REQUIRE(net && pts && labels && npairs > 0, "null argument or empty batch");
  REQUIRE(npairs <= kMaxPairs, "too many pairs (%zu)", npairs);
  const auto b = posenet::batch(ctx, net, static_cast<int>(npairs), true);
  h2d(ctx, b.pts, pts, 2 * npairs * posenet::kPts * 16);
  h2d(ctx, b.labels, labels, npairs * posenet::kOut * 4);
  posenet::encode(ctx, net, b, true);
  posenet::head_forward(ctx, net, b);
  posenet::loss_backward(ctx, net, b);
  d2h(ctx, loss, b.loss, 4);
  d2h(ctx, grads, net->grad, posenet::kParams * 4);
  posenet::check_error(ctx, net);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_train_step(lcr_ctx* ctx, lcr_posenet* net, const lcr_cloud* const* src,
                                  const lcr_cloud* const* tgt, const float* transforms, size_t npairs, uint64_t seed,
                                  const lcr_adamw_params* opt, float* loss) {
  API_BEGIN(ctx)
  REQUIRE(net && src && tgt && transforms && opt && npairs > 0, "null argument or empty batch");
  REQUIRE(npairs <= kMaxPairs, "too many pairs (%zu)", npairs);
  REQUIRE(opt->lr >= 0.f && opt->beta1 >= 0.f && opt->beta1 < 1.f && opt->beta2 >= 0.f && opt->beta2 < 1.f &&
              opt->eps > 0.f && opt->weight_decay >= 0.f,
          "bad AdamW parameters");
  const auto refs = cloud_refs(src, tgt, npairs);
  const auto b = posenet::batch(ctx, net, static_cast<int>(npairs), true);
  h2d(ctx, b.refs, refs.data(), refs.size() * sizeof(posenet::CloudRef));
  h2d(ctx, b.guess, transforms, npairs * 16 * 4);
  posenet::sample(ctx, b.refs, static_cast<int>(2 * npairs), seed, b.pts, b.cen);
  posenet::labels_from_poses(ctx, b, b.guess);
  posenet::encode(ctx, net, b, true);
  posenet::head_forward(ctx, net, b);
  posenet::loss_backward(ctx, net, b);
  posenet::adamw(ctx, net, opt);
  d2h(ctx, loss, b.loss, 4);
  posenet::check_error(ctx, net);
  API_END(ctx)
  return LCR_OK;
}

lcr_status lcr_posenet_propose(lcr_ctx* ctx, lcr_posenet* net, const lcr_cloud* const* src,
                               const lcr_cloud* const* tgt, size_t npairs, uint64_t seed, float* guesses) {
  API_BEGIN(ctx)
  REQUIRE(net && (npairs == 0 || (src && tgt && guesses)), "null argument");
  REQUIRE(npairs <= kMaxPairs, "too many pairs (%zu)", npairs);
  if (npairs) {
    const auto refs = cloud_refs(src, tgt, npairs);
    const auto b = posenet::batch(ctx, net, static_cast<int>(npairs), false);
    h2d(ctx, b.refs, refs.data(), refs.size() * sizeof(posenet::CloudRef));
    posenet::sample(ctx, b.refs, static_cast<int>(2 * npairs), seed, b.pts, b.cen);
    posenet::encode(ctx, net, b, false);
    posenet::head_forward(ctx, net, b);
    posenet::poses(ctx, b);
    d2h(ctx, guesses, b.guess, npairs * 16 * 4);
    posenet::check_error(ctx, net);
  }
  API_END(ctx)
  return LCR_OK;
}

}  // extern "C"
