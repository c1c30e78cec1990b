// Autotuning of launch shapes: warps per block of the unordered k-NN kernels
// (StatisticalOutlierRemoval, NormalEstimation) and persistent blocks per SM
// of the batched ICP kernels.  Every result of the library is independent of
// these shapes (per-query outputs, fixed-order reductions); only the speed
// changes, and the best shape depends on the cloud size and the device.
//
// lcr_autotune times each candidate on a representative pair with CUDA events
// (one untimed run, then the median of three), applies the fastest, and can
// record the choice in a cache file: one JSON object per line keyed by the
// device name, its SM count and the source's size class (floor(log2 n)).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

#include "lcr_internal.cuh"

namespace {

std::string tune_key(lcr_ctx* ctx, size_t n) {
  cudaDeviceProp prop;
  CUDA_TRY(cudaGetDeviceProperties(&prop, ctx->device));
  const int cls = n > 0 ? static_cast<int>(std::floor(std::log2(static_cast<double>(n)))) : 0;
  char b[384];
  snprintf(b, sizeof b, "%s|%d SMs|n=2^%d", prop.name, prop.multiProcessorCount, cls);
  return b;
}

bool valid(const lcr_tune& t) {
  return t.sor_warps >= 1 && t.sor_warps <= 8 && t.normals_warps >= 1 && t.normals_warps <= 8 &&
         t.icp_blocks_per_sm >= 1 && t.icp_blocks_per_sm <= 8;
}

int field(const std::string& line, const char* name, bool& ok) {
  const std::string tag = std::string("\"") + name + "\": ";
  const size_t p = line.find(tag);
  if (p == std::string::npos) {
    ok = false;
    return 0;
  }
  return std::atoi(line.c_str() + p + tag.size());
}

// The last record with this key wins.
bool cache_lookup(const char* path, const std::string& key, lcr_tune* out) {
  std::ifstream f(path);
  if (!f) return false;
  const std::string tag = "\"key\": \"" + key + "\"";
  std::string line;
  bool found = false;
  while (std::getline(f, line)) {
    if (line.find(tag) == std::string::npos) continue;
    bool ok = true;
    lcr_tune t;
    t.sor_warps = field(line, "sor_warps", ok);
    t.normals_warps = field(line, "normals_warps", ok);
    t.icp_blocks_per_sm = field(line, "icp_blocks_per_sm", ok);
    if (ok && valid(t)) {
      *out = t;
      found = true;
    }
  }
  return found;
}

void cache_store(const char* path, const std::string& key, const lcr_tune& t) {
  std::ofstream f(path, std::ios::app);
  if (!f) LCR_THROW(LCR_ERR_IO, "cannot append to the tuning cache %s", path);
  f << "{\"key\": \"" << key << "\", \"sor_warps\": " << t.sor_warps << ", \"normals_warps\": " << t.normals_warps
    << ", \"icp_blocks_per_sm\": " << t.icp_blocks_per_sm << "}\n";
}

double median3(double a, double b, double c) { return std::max(std::min(a, b), std::min(std::max(a, b), c)); }

// One untimed run, then the median of three timed ones.
template <class F>
double time_median(F&& once) {
  once();
  double t[3];
  for (double& v : t) v = once();
  return median3(t[0], t[1], t[2]);
}

}  // namespace

void tune_apply(lcr_ctx* ctx, const lcr_tune& t) {
  if (!valid(t)) LCR_THROW(LCR_ERR_INVALID_ARG, "launch shapes out of range (1-8)");
  const bool icp_changed = t.icp_blocks_per_sm != ctx->tune.icp_bps;
  ctx->tune.sor_warps = t.sor_warps;
  ctx->tune.ne_warps = t.normals_warps;
  ctx->tune.icp_bps = t.icp_blocks_per_sm;
  if (icp_changed) icp_graphs_reset(ctx);
}

lcr_tune tune_current(const lcr_ctx* ctx) {
  lcr_tune t;
  t.sor_warps = ctx->tune.sor_warps;
  t.normals_warps = ctx->tune.ne_warps;
  t.icp_blocks_per_sm = ctx->tune.icp_bps;
  return t;
}

void autotune_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const char* cache_path,
                  lcr_tune_report* rep) {
  std::memset(rep, 0, sizeof(*rep));
  const std::string key = tune_key(ctx, src->n);
  lcr_tune cached;
  if (cache_path && cache_lookup(cache_path, key, &cached)) {
    tune_apply(ctx, cached);
    rep->chosen = cached;
    rep->from_cache = 1;
    return;
  }
  const bool was_timing = ctx->timing;
  ctx->timing = true;
  lcr_tune best = tune_current(ctx);
  try {
    kernel_time_take(ctx, LCR_KT_SOR_KNN);
    kernel_time_take(ctx, LCR_KT_NORMALS_KNN);
    // StatisticalOutlierRemoval k-NN (k = 50, the tools' default)
    double best_ms = INFINITY;
    for (int w : {2, 3, 4, 5, 6, 8}) {
      ctx->tune.sor_warps = w;
      const double ms = time_median([&] {
        lcr_sor_stats st;
        sor_run(ctx, src, 50, 1.0, nullptr, nullptr, &st, nullptr);
        return kernel_time_take(ctx, LCR_KT_SOR_KNN);
      });
      rep->sor_ms[w - 1] = ms;
      if (ms < best_ms) {
        best_ms = ms;
        best.sor_warps = w;
      }
    }
    ctx->tune.sor_warps = best.sor_warps;
    // NormalEstimation k-NN (k = 30)
    best_ms = INFINITY;
    const float vp[3] = {0.f, 0.f, 0.f};
    for (int w : {2, 3, 4, 5, 6, 8}) {
      ctx->tune.ne_warps = w;
      const double ms = time_median([&] {
        cloud_release(ctx, normals_run(ctx, src, 30, vp, 0));
        return kernel_time_take(ctx, LCR_KT_NORMALS_KNN);
      });
      rep->normals_ms[w - 1] = ms;
      if (ms < best_ms) {
        best_ms = ms;
        best.normals_warps = w;
      }
    }
    ctx->tune.ne_warps = best.normals_warps;
    // batched ICP persistent grid: point-to-point ICP of src onto tgt
    lcr_icp_params p;
    lcr_icp_params_default(&p);
    p.max_correspondence_distance = 0.05;
    p.max_iterations = 20;
    p.compute_fitness = 0;
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    best_ms = INFINITY;
    for (int bps : {2, 3, 4, 6, 8}) {
      if (bps != ctx->tune.icp_bps) {
        ctx->tune.icp_bps = bps;
        icp_graphs_reset(ctx);
      }
      const double ms = time_median([&] {
        lcr_icp_result res;
        CUDA_TRY(cudaEventRecord(a, ctx->stream));
        icp_run(ctx, src, tgt, &p, nullptr, &res);
        CUDA_TRY(cudaEventRecord(b, ctx->stream));
        CUDA_TRY(cudaEventSynchronize(b));
        float v = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&v, a, b));
        return static_cast<double>(v);
      });
      rep->icp_ms[bps - 1] = ms;
      if (ms < best_ms) {
        best_ms = ms;
        best.icp_blocks_per_sm = bps;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  } catch (...) {
    ctx->timing = was_timing;
    throw;
  }
  ctx->timing = was_timing;
  tune_apply(ctx, best);
  rep->chosen = best;
  if (cache_path) cache_store(cache_path, key, best);
}
