// Context, device memory, cloud storage and the elementwise cloud kernels
// (pack/unpack of PCL records, rigid transform with normals, centroid).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "lcr_internal.cuh"

// ------------------------------------------------------------------ memory
void* dev_alloc(lcr_ctx* ctx, size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) bytes = 16;
  CUDA_TRY(cudaMallocAsync(&p, bytes, ctx->stream));
  return p;
}

void dev_free(lcr_ctx* ctx, void* p) {
  if (p) CUDA_TRY(cudaFreeAsync(p, ctx->stream));
}

KernelTimer::KernelTimer(lcr_ctx* c, int w) : ctx(c), which(w) {
  if (!ctx->timing) return;
  for (cudaEvent_t* e : {&a, &b}) {
    if (!ctx->event_pool.empty()) {
      *e = ctx->event_pool.back();
      ctx->event_pool.pop_back();
    } else {
      CUDA_TRY(cudaEventCreate(e));
    }
  }
  CUDA_TRY(cudaEventRecord(a, ctx->stream));
}

KernelTimer::~KernelTimer() {
  if (!a) return;
  cudaEventRecord(b, ctx->stream);
  ctx->kt[which].pending.emplace_back(a, b);
}

void* pinned(lcr_ctx* ctx, size_t bytes) {
  if (bytes > ctx->pinned_bytes) {
    sync(ctx);
    if (ctx->pinned) CUDA_TRY(cudaFreeHost(ctx->pinned));
    ctx->pinned = nullptr;
    const size_t want = std::max<size_t>(bytes, 1 << 16);
    CUDA_TRY(cudaMallocHost(&ctx->pinned, want));
    ctx->pinned_bytes = want;
  }
  return ctx->pinned;
}

void sync(lcr_ctx* ctx) { CUDA_TRY(cudaStreamSynchronize(ctx->stream)); }

lcr_cloud* cloud_alloc(lcr_ctx* ctx, size_t n) {
  lcr_cloud* c = new lcr_cloud();
  c->n = n;
  const size_t m = std::max<size_t>(n, 1);
  char* blk = static_cast<char*>(dev_alloc(ctx, m * (16 + 16 + 4) + 512));
  c->xyz = reinterpret_cast<float4*>(blk);
  c->nrm = reinterpret_cast<float4*>(blk + m * 16);
  c->rgb = reinterpret_cast<uint32_t*>(blk + m * 32);
  return c;
}

void cloud_release(lcr_ctx* ctx, lcr_cloud* c) {
  if (!c) return;
  free_index(ctx, c->index);
  if (c->nbr) {
    dev_free(ctx, c->nbr->block);
    delete c->nbr;
  }
  if (c->graph) {
    dev_free(ctx, c->graph->rows);
    delete c->graph;
  }
  dev_free(ctx, c->xyz);
  delete c;
}

const Index& cloud_index(lcr_ctx* ctx, const lcr_cloud* c) {
  if (!c->index) const_cast<lcr_cloud*>(c)->index = build_index(ctx, c->xyz, static_cast<int>(c->n));
  return *c->index;
}

// ----------------------------------------------------------------- kernels
namespace {

struct __align__(16) Sum4 {
  double x, y, z, w;
};

// lcr_point (48 B) = float4 {x y z _} + float4 {nx ny nz _} + float4 {rgba curvature _ _}
__global__ void k_unpack(const float4* __restrict__ rec, size_t n, float4* __restrict__ xyz, float4* __restrict__ nrm,
                         uint32_t* __restrict__ rgb) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = rec[3 * i], b = rec[3 * i + 1], c = rec[3 * i + 2];
  xyz[i] = make_float4(a.x, a.y, a.z, 0.f);
  nrm[i] = make_float4(b.x, b.y, b.z, c.y);
  rgb[i] = __float_as_uint(c.x);
}

__global__ void k_pack(const float4* __restrict__ xyz, const float4* __restrict__ nrm, const uint32_t* __restrict__ rgb,
                       size_t n, float4* __restrict__ rec) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i], q = nrm[i];
  rec[3 * i] = make_float4(p.x, p.y, p.z, 1.f);
  rec[3 * i + 1] = make_float4(q.x, q.y, q.z, 0.f);
  rec[3 * i + 2] = make_float4(__uint_as_float(rgb[i]), q.w, 0.f, 0.f);
}

__global__ void k_from_xyz(const float* __restrict__ in, size_t n, float4* __restrict__ xyz, float4* __restrict__ nrm,
                           uint32_t* __restrict__ rgb) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  xyz[i] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.f);
  nrm[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  rgb[i] = 0u;
}

// transformPointCloudWithNormals: p' = M p (x,y,z,1), n' = M3x3 n; non-finite
// points are copied unchanged.
__global__ void k_transform(const float4* __restrict__ xyz, const float4* __restrict__ nrm,
                            const uint32_t* __restrict__ rgb, size_t n, Xf T, float4* __restrict__ oxyz,
                            float4* __restrict__ onrm, uint32_t* __restrict__ orgb) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i], q = nrm[i];
  float4 op = p, oq = q;
  if (finite3(p.x, p.y, p.z)) {
    const float3 a = xf_apply(T, p.x, p.y, p.z);
    const float3 b = xf_rotate(T, q.x, q.y, q.z);
    op = make_float4(a.x, a.y, a.z, 0.f);
    oq = make_float4(b.x, b.y, b.z, q.w);
  }
  oxyz[i] = op;
  onrm[i] = oq;
  orgb[i] = rgb[i];
}

// FP64 centroid: per-block partial sums (x, y, z, count) then one block adds the
// partials in block order (deterministic).
__global__ void k_centroid_partial(const float4* __restrict__ xyz, size_t n, Sum4* __restrict__ part) {
  __shared__ Sum4 ws[8];
  double sx = 0, sy = 0, sz = 0, c = 0;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const float4 p = xyz[i];
    if (!finite3(p.x, p.y, p.z)) continue;
    sx += p.x; sy += p.y; sz += p.z; c += 1.0;
  }
  sx = warp_sum(sx); sy = warp_sum(sy); sz = warp_sum(sz); c = warp_sum(c);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = Sum4{sx, sy, sz, c};
  __syncthreads();
  if (threadIdx.x == 0) {
    Sum4 s = Sum4{0, 0, 0, 0};
    for (int j = 0; j < static_cast<int>(blockDim.x >> 5); ++j) {
      s.x += ws[j].x; s.y += ws[j].y; s.z += ws[j].z; s.w += ws[j].w;
    }
    part[blockIdx.x] = s;
  }
}

// Sum of the block partials, one warp: lane l adds partials l, l+32, ... in
// order, then a fixed shuffle tree.  out4 = (mean xyz, count) in FP64; outf
// (may be null) receives the mean as float.
__global__ void k_centroid_final(const Sum4* __restrict__ part, int nb, double* __restrict__ out,
                                 float* __restrict__ outf) {
  const int lane = threadIdx.x;
  double x = 0, y = 0, z = 0, w = 0;
  for (int j = lane; j < nb; j += 32) {
    const Sum4 p = part[j];
    x += p.x; y += p.y; z += p.z; w += p.w;
  }
  x = warp_sum(x); y = warp_sum(y); z = warp_sum(z); w = warp_sum(w);
  if (lane != 0) return;
  const double c = w > 0 ? w : 1.0;
  out[0] = x / c;
  out[1] = y / c;
  out[2] = z / c;
  out[3] = w;
  if (outf) {
    outf[0] = static_cast<float>(out[0]);
    outf[1] = static_cast<float>(out[1]);
    outf[2] = static_cast<float>(out[2]);
  }
}

}  // namespace

lcr_cloud* upload_records(lcr_ctx* ctx, const void* recs, size_t n, bool device_src) {
  lcr_cloud* c = cloud_alloc(ctx, n);
  if (n == 0) return c;
  float4* tmp = nullptr;
  const float4* src = static_cast<const float4*>(recs);
  if (!device_src) {
    tmp = static_cast<float4*>(dev_alloc(ctx, n * sizeof(lcr_point)));
    CUDA_TRY(cudaMemcpyAsync(tmp, recs, n * sizeof(lcr_point), cudaMemcpyHostToDevice, ctx->stream));
    src = tmp;
  }
  LCR_LAUNCH(ctx, k_unpack, static_cast<unsigned>((n + 255) / 256), 256, 0, src, n, c->xyz, c->nrm, c->rgb);
  dev_free(ctx, tmp);
  return c;
}

lcr_cloud* upload_xyz(lcr_ctx* ctx, const float* xyz, size_t n) {
  lcr_cloud* c = cloud_alloc(ctx, n);
  if (n == 0) return c;
  float* tmp = static_cast<float*>(dev_alloc(ctx, n * 3 * sizeof(float)));
  CUDA_TRY(cudaMemcpyAsync(tmp, xyz, n * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  LCR_LAUNCH(ctx, k_from_xyz, static_cast<unsigned>((n + 255) / 256), 256, 0, tmp, n, c->xyz, c->nrm, c->rgb);
  dev_free(ctx, tmp);
  return c;
}

void download_records(lcr_ctx* ctx, const lcr_cloud* c, void* out) {
  if (c->n == 0) return;
  float4* tmp = static_cast<float4*>(dev_alloc(ctx, c->n * sizeof(lcr_point)));
  LCR_LAUNCH(ctx, k_pack, static_cast<unsigned>((c->n + 255) / 256), 256, 0, c->xyz, c->nrm, c->rgb, c->n, tmp);
  CUDA_TRY(cudaMemcpyAsync(out, tmp, c->n * sizeof(lcr_point), cudaMemcpyDeviceToHost, ctx->stream));
  dev_free(ctx, tmp);
  sync(ctx);
}

lcr_cloud* concat_clouds(lcr_ctx* ctx, const lcr_cloud* a, const lcr_cloud* b) {
  lcr_cloud* c = cloud_alloc(ctx, a->n + b->n);
  if (a->n) {
    CUDA_TRY(cudaMemcpyAsync(c->xyz, a->xyz, a->n * 16, cudaMemcpyDeviceToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(c->nrm, a->nrm, a->n * 16, cudaMemcpyDeviceToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(c->rgb, a->rgb, a->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  if (b->n) {
    CUDA_TRY(cudaMemcpyAsync(c->xyz + a->n, b->xyz, b->n * 16, cudaMemcpyDeviceToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(c->nrm + a->n, b->nrm, b->n * 16, cudaMemcpyDeviceToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(c->rgb + a->n, b->rgb, b->n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return c;
}

lcr_cloud* transform_run(lcr_ctx* ctx, const lcr_cloud* in, const float* m) {
  lcr_cloud* c = cloud_alloc(ctx, in->n);
  if (in->n == 0) return c;
  Xf T;
  for (int i = 0; i < 12; ++i) T.m[i] = m[i];
  LCR_LAUNCH(ctx, k_transform, static_cast<unsigned>((in->n + 255) / 256), 256, 0, in->xyz, in->nrm, in->rgb, in->n,
             T, c->xyz, c->nrm, c->rgb);
  return c;
}

void centroid_device(lcr_ctx* ctx, const lcr_cloud* in, double* out4, float* outf) {
  const int nb = std::max(1, std::min(ctx->sms * 2, static_cast<int>((in->n + 255) / 256)));
  Sum4* part = static_cast<Sum4*>(dev_alloc(ctx, nb * sizeof(Sum4)));
  LCR_LAUNCH(ctx, k_centroid_partial, nb, 256, 0, in->xyz, in->n, part);
  LCR_LAUNCH(ctx, k_centroid_final, 1, 32, 0, part, nb, out4, outf);
  dev_free(ctx, part);
}

void centroid_run(lcr_ctx* ctx, const lcr_cloud* in, double* c4) {
  double* out = static_cast<double*>(dev_alloc(ctx, 4 * sizeof(double)));
  centroid_device(ctx, in, out, nullptr);
  double* h = static_cast<double*>(pinned(ctx, 4 * sizeof(double)));
  CUDA_TRY(cudaMemcpyAsync(h, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  dev_free(ctx, out);
  sync(ctx);
  for (int i = 0; i < 4; ++i) c4[i] = h[i];
}

double kernel_time_take(lcr_ctx* ctx, int which) {
  sync(ctx);
  auto& t = ctx->kt[which];
  double ms = t.ms;
  for (auto& e : t.pending) {
    float v = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&v, e.first, e.second));
    ms += v;
    ctx->event_pool.push_back(e.first);
    ctx->event_pool.push_back(e.second);
  }
  t.pending.clear();
  t.ms = 0.0;
  t.launches = 0;
  return ms;
}
