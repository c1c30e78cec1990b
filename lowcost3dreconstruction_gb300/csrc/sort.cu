// Data-movement primitives: stable LSD radix sort, order-preserving compaction,
// row gathers and bounding boxes.  All HBM-bound integer work on the context
// stream; no library calls.
#include <algorithm>

#include "lcr_internal.cuh"

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;                      // rounds of 256 per tile
constexpr int kSortTile = kSortThreads * kSortItems;  // 2048 keys per block

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Per-block digit histogram, written block-major: hist[b * 256 + d].
__global__ void k_radix_hist(const uint32_t* __restrict__ keys, int n, int shift, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = static_cast<size_t>(blockIdx.x) * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i = base + r * kSortThreads + threadIdx.x;
    if (i < static_cast<size_t>(n)) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[static_cast<size_t>(blockIdx.x) * 256 + threadIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m counters (block counts of a compaction: m is small) by a
// single block of 1024 threads, each owning a contiguous chunk.  total (may be
// null) receives the sum.
__global__ void k_scan_exclusive(uint32_t* __restrict__ a, int m, uint32_t* __restrict__ total) {
  __shared__ uint32_t warp_sums[32];
  const int t = threadIdx.x;
  const int chunk = (m + blockDim.x - 1) / blockDim.x;
  const int b = t * chunk, e = min(m, b + chunk);
  uint32_t s = 0;
  for (int i = b; i < e; ++i) s += a[i];
  // block exclusive scan of s
  const int lane = t & 31, w = t >> 5;
  uint32_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(LCR_FULL, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t ws = lane < static_cast<int>(blockDim.x >> 5) ? warp_sums[lane] : 0;
    uint32_t wi = ws;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(LCR_FULL, wi, o);
      if (lane >= o) wi += v;
    }
    warp_sums[lane] = wi - ws;
    if (lane == 31 && total) *total = wi;
  }
  __syncthreads();
  uint32_t run = warp_sums[w] + incl - s;
  for (int i = b; i < e; ++i) {
    const uint32_t v = a[i];
    a[i] = run;
    run += v;
  }
}

// Per-digit exclusive scan over the blocks, one block per digit (column d of
// the block-major histogram), in place; totals[d] = number of keys with digit d.
__global__ void k_radix_offsets(uint32_t* __restrict__ hist, int nblk, uint32_t* __restrict__ totals) {
  __shared__ uint32_t s_wsum[kSortThreads / 32];
  const int d = blockIdx.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
  uint32_t carry = 0;
  for (int j0 = 0; j0 < nblk; j0 += kSortThreads) {
    const int j = j0 + t;
    const uint32_t v = j < nblk ? hist[static_cast<size_t>(j) * 256 + d] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(LCR_FULL, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) s_wsum[w] = incl;
    __syncthreads();
    uint32_t wbase = 0, all = 0;
#pragma unroll
    for (int k = 0; k < kSortThreads / 32; ++k) {
      wbase += k < w ? s_wsum[k] : 0u;
      all += s_wsum[k];
    }
    if (j < nblk) hist[static_cast<size_t>(j) * 256 + d] = carry + wbase + incl - v;
    carry += all;
    __syncthreads();
  }
  if (t == 0) totals[d] = carry;
}

// Stable scatter.  Each block's output base for digit d is the exclusive sum of
// the digit totals below d plus its own per-digit prefix.  Elements are ranked
// round by round (256 at a time, in input order): within a warp by
// __match_any_sync peers below the lane, across warps by a per-digit prefix
// over warp counts, across rounds by a running per-digit base.
__global__ void k_radix_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int n, int shift,
                                const uint32_t* __restrict__ hist, const uint32_t* __restrict__ totals) {
  __shared__ uint32_t s_off[256];
  __shared__ uint32_t s_w[kSortThreads / 32][256];
  __shared__ uint32_t s_wsum[kSortThreads / 32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  {
    const uint32_t total = totals[t];
    uint32_t incl = total;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(LCR_FULL, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) s_wsum[w] = incl;
    __syncthreads();
    uint32_t wbase = 0;
#pragma unroll
    for (int k = 0; k < kSortThreads / 32; ++k) wbase += k < w ? s_wsum[k] : 0u;
    s_off[t] = wbase + incl - total + hist[static_cast<size_t>(blockIdx.x) * 256 + t];
  }
#pragma unroll
  for (int j = 0; j < kSortThreads / 32; ++j) s_w[j][t] = 0;
  __syncthreads();
  const size_t base = static_cast<size_t>(blockIdx.x) * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
    const size_t i = base + r * kSortThreads + t;
    const bool valid = i < static_cast<size_t>(n);
    const uint32_t k = valid ? kin[i] : 0u;
    const uint32_t v = valid ? vin[i] : 0u;
    const uint32_t d = (k >> shift) & 255u;
    const unsigned peers = __match_any_sync(LCR_FULL, valid ? d : 0x100u);
    const uint32_t rank = __popc(peers & lanemask_lt());
    const bool leader = (__ffs(peers) - 1) == lane;
    if (valid && leader) s_w[w][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = s_off[t];
#pragma unroll
      for (int j = 0; j < kSortThreads / 32; ++j) {
        const uint32_t c = s_w[j][t];
        s_w[j][t] = run;
        run += c;
      }
      s_off[t] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_w[w][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortThreads / 32; ++j) s_w[j][t] = 0;
    __syncthreads();
  }
}

// ---------------------------------------------------------------- compaction
constexpr int kCompThreads = 256;
constexpr int kCompItems = 8;
constexpr int kCompTile = kCompThreads * kCompItems;

__global__ void k_flag_count(const uint8_t* __restrict__ flags, int n, uint32_t* __restrict__ cnt) {
  __shared__ uint32_t ws[kCompThreads / 32];
  const size_t base = static_cast<size_t>(blockIdx.x) * kCompTile;
  uint32_t c = 0;
#pragma unroll
  for (int r = 0; r < kCompItems; ++r) {
    const size_t i = base + r * kCompThreads + threadIdx.x;
    c += (i < static_cast<size_t>(n) && flags[i]) ? 1u : 0u;
  }
  c = warp_sum(c);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int j = 0; j < kCompThreads / 32; ++j) s += ws[j];
    cnt[blockIdx.x] = s;
  }
}

__global__ void k_flag_scatter(const uint8_t* __restrict__ flags, int n, const uint32_t* __restrict__ offs,
                               uint32_t* __restrict__ out) {
  __shared__ uint32_t ws[kCompThreads / 32];
  __shared__ uint32_t s_base;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) s_base = offs[blockIdx.x];
  __syncthreads();
  const size_t base = static_cast<size_t>(blockIdx.x) * kCompTile;
  for (int r = 0; r < kCompItems; ++r) {
    const size_t i = base + r * kCompThreads + t;
    const bool f = i < static_cast<size_t>(n) && flags[i];
    const unsigned m = __ballot_sync(LCR_FULL, f);
    if (lane == 0) ws[w] = __popc(m);
    __syncthreads();
    uint32_t before = s_base;
    for (int j = 0; j < w; ++j) before += ws[j];
    if (f) out[before + __popc(m & lanemask_lt())] = static_cast<uint32_t>(i);
    __syncthreads();
    if (t == 0) {
      uint32_t s = 0;
      for (int j = 0; j < kCompThreads / 32; ++j) s += ws[j];
      s_base += s;
    }
    __syncthreads();
  }
}

__global__ void k_gather_cloud(const float4* __restrict__ xyz, const float4* __restrict__ nrm,
                               const uint32_t* __restrict__ rgb, const uint32_t* __restrict__ idx, int n,
                               float4* __restrict__ oxyz, float4* __restrict__ onrm, uint32_t* __restrict__ orgb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t i = idx[j];
  oxyz[j] = xyz[i];
  onrm[j] = nrm[i];
  orgb[j] = rgb[i];
}

// Ordered-integer encoding of floats for atomic min/max.
__device__ __forceinline__ uint32_t f2o(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

__global__ void k_bbox_init(uint32_t* b) {
  if (threadIdx.x < 3) {
    b[threadIdx.x] = f2o(__int_as_float(0x7f800000));
    b[3 + threadIdx.x] = f2o(-__int_as_float(0x7f800000));
  }
}

__global__ void k_bbox(const float4* __restrict__ xyz, int n, uint32_t* __restrict__ b) {
  float lx = __int_as_float(0x7f800000), ly = lx, lz = lx, hx = -lx, hy = -lx, hz = -lx;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = xyz[i];
    if (!finite3(p.x, p.y, p.z)) continue;
    lx = fminf(lx, p.x); ly = fminf(ly, p.y); lz = fminf(lz, p.z);
    hx = fmaxf(hx, p.x); hy = fmaxf(hy, p.y); hz = fmaxf(hz, p.z);
  }
  lx = warp_min(lx); ly = warp_min(ly); lz = warp_min(lz);
  hx = warp_max(hx); hy = warp_max(hy); hz = warp_max(hz);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&b[0], f2o(lx)); atomicMin(&b[1], f2o(ly)); atomicMin(&b[2], f2o(lz));
    atomicMax(&b[3], f2o(hx)); atomicMax(&b[4], f2o(hy)); atomicMax(&b[5], f2o(hz));
  }
}

__global__ void k_bbox_finish(const uint32_t* b, float4* out) {
  if (threadIdx.x == 0) {
    out[0] = make_float4(o2f(b[0]), o2f(b[1]), o2f(b[2]), 0.f);
    out[1] = make_float4(o2f(b[3]), o2f(b[4]), o2f(b[5]), 0.f);
  }
}

}  // namespace

void radix_sort_pairs(lcr_ctx* ctx, uint32_t* keys, uint32_t* vals, int n, int bits) {
  if (n <= 1) return;
  const int nblk = (n + kSortTile - 1) / kSortTile;
  uint32_t* tk = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * static_cast<size_t>(n)));
  uint32_t* tv = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * static_cast<size_t>(n)));
  uint32_t* hist = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * 256 * (static_cast<size_t>(nblk) + 1)));
  uint32_t* totals = hist + 256 * static_cast<size_t>(nblk);
  uint32_t *ki = keys, *vi = vals, *ko = tk, *vo = tv;
  const int passes = (std::max(bits, 1) + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    LCR_LAUNCH(ctx, k_radix_hist, nblk, kSortThreads, 0, ki, n, shift, hist);
    LCR_LAUNCH(ctx, k_radix_offsets, 256, kSortThreads, 0, hist, nblk, totals);
    LCR_LAUNCH(ctx, k_radix_scatter, nblk, kSortThreads, 0, ki, vi, ko, vo, n, shift, hist, totals);
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  if (ki != keys) {
    CUDA_TRY(cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(vals, vi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  dev_free(ctx, tk);
  dev_free(ctx, tv);
  dev_free(ctx, hist);
}

// Writes the count to *count_dev (may be null); no host synchronisation.
void compact_flags_async(lcr_ctx* ctx, const uint8_t* flags, int n, uint32_t* out_idx, uint32_t* count_dev) {
  if (n <= 0) return;
  const int nblk = (n + kCompTile - 1) / kCompTile;
  uint32_t* cnt = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * (nblk + 1)));
  LCR_LAUNCH(ctx, k_flag_count, nblk, kCompThreads, 0, flags, n, cnt);
  LCR_LAUNCH(ctx, k_scan_exclusive, 1, 1024, 0, cnt, nblk, count_dev ? count_dev : cnt + nblk);
  LCR_LAUNCH(ctx, k_flag_scatter, nblk, kCompThreads, 0, flags, n, cnt, out_idx);
  dev_free(ctx, cnt);
}

int compact_flags(lcr_ctx* ctx, const uint8_t* flags, int n, uint32_t* out_idx) {
  if (n <= 0) return 0;
  uint32_t* d = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t)));
  compact_flags_async(ctx, flags, n, out_idx, d);
  uint32_t* h = static_cast<uint32_t*>(pinned(ctx, sizeof(uint32_t)));
  CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  dev_free(ctx, d);
  sync(ctx);
  return static_cast<int>(*h);
}

void gather_cloud(lcr_ctx* ctx, const lcr_cloud* in, const uint32_t* idx, int n, lcr_cloud* out) {
  if (n <= 0) return;
  LCR_LAUNCH(ctx, k_gather_cloud, (n + 255) / 256, 256, 0, in->xyz, in->nrm, in->rgb, idx, n, out->xyz, out->nrm,
             out->rgb);
}

void bbox(lcr_ctx* ctx, const float4* xyz, int n, float4* out2) {
  uint32_t* b = static_cast<uint32_t*>(dev_alloc(ctx, 8 * sizeof(uint32_t)));
  LCR_LAUNCH(ctx, k_bbox_init, 1, 32, 0, b);
  if (n > 0) {
    const int grid = std::min((n + 255) / 256, ctx->sms * 4);
    LCR_LAUNCH(ctx, k_bbox, grid, 256, 0, xyz, n, b);
  }
  LCR_LAUNCH(ctx, k_bbox_finish, 1, 32, 0, b, out2);
  dev_free(ctx, b);
}
