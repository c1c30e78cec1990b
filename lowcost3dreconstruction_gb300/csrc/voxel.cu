// pcl::VoxelGrid as sort-and-segment (pcl_tools/cloud_downsampling.cpp:73-76).
//
// PCL semantics restated: bounding box of the finite points; inverse leaf
// 1/leaf in float; refuse (output = input) when the voxel count overflows
// int32; per point ijk = int(floor(p*inv) - float(min_b)) and
// idx = i + j*div_x + k*div_x*div_y; one output point per occupied voxel in
// ascending idx order, every field the float mean of its members.  The stable
// radix sort fixes the within-voxel summation order to ascending input index.
#include <algorithm>

#include "lcr_internal.cuh"

namespace {

struct VoxelSetup {
  float inv[3];
  int min_b[3];
  int div_b[3];
  int overflow;
  int empty;
};

__global__ void k_voxel_setup(const float4* __restrict__ box, float lx, float ly, float lz, VoxelSetup* s) {
  if (threadIdx.x != 0) return;
  const float4 lo = box[0], hi = box[1];
  const float leaf[3] = {lx, ly, lz};
  const float l3[3] = {lo.x, lo.y, lo.z}, h3[3] = {hi.x, hi.y, hi.z};
  VoxelSetup v;
  v.empty = !(lo.x <= hi.x);
  v.overflow = 0;
  long long d[3] = {1, 1, 1};
  for (int a = 0; a < 3; ++a) {
    v.inv[a] = __fdiv_rn(1.0f, leaf[a]);
    v.min_b[a] = 0;
    v.div_b[a] = 1;
  }
  if (!v.empty) {
    for (int a = 0; a < 3; ++a) {
      const float cells = __fmul_rn(__fsub_rn(h3[a], l3[a]), v.inv[a]);
      if (!(cells < 9.0e18f)) {
        v.overflow = 1;
        continue;
      }
      d[a] = static_cast<long long>(cells) + 1;
    }
    if (!v.overflow) {
      const double prod = static_cast<double>(d[0]) * static_cast<double>(d[1]) * static_cast<double>(d[2]);
      if (prod > 2147483647.0 || d[0] * d[1] * d[2] > 2147483647LL) v.overflow = 1;
    }
    if (!v.overflow) {
      for (int a = 0; a < 3; ++a) {
        v.min_b[a] = static_cast<int>(floorf(__fmul_rn(l3[a], v.inv[a])));
        const int max_b = static_cast<int>(floorf(__fmul_rn(h3[a], v.inv[a])));
        v.div_b[a] = max_b - v.min_b[a] + 1;
      }
    }
  }
  *s = v;
}

__global__ void k_voxel_keys(const float4* __restrict__ xyz, int n, const VoxelSetup* __restrict__ s,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i];
  uint32_t key = 0xffffffffu;
  if (!s->overflow && !s->empty && finite3(p.x, p.y, p.z)) {
    const int i0 = static_cast<int>(__fsub_rn(floorf(__fmul_rn(p.x, s->inv[0])), static_cast<float>(s->min_b[0])));
    const int i1 = static_cast<int>(__fsub_rn(floorf(__fmul_rn(p.y, s->inv[1])), static_cast<float>(s->min_b[1])));
    const int i2 = static_cast<int>(__fsub_rn(floorf(__fmul_rn(p.z, s->inv[2])), static_cast<float>(s->min_b[2])));
    key = static_cast<uint32_t>(i0 + i1 * s->div_b[0] + i2 * (s->div_b[0] * s->div_b[1]));
  }
  keys[i] = key;
  vals[i] = static_cast<uint32_t>(i);
}

__global__ void k_segment_heads(const uint32_t* __restrict__ keys, int n, uint8_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = keys[i];
  flags[i] = (k != 0xffffffffu && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
}

// One thread per voxel: sequential FP32 sums in sorted order, IEEE division.
__global__ void k_voxel_centroids(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int n,
                                  const uint32_t* __restrict__ starts, int nseg, const float4* __restrict__ xyz,
                                  const float4* __restrict__ nrm, const uint32_t* __restrict__ rgb,
                                  float4* __restrict__ oxyz, float4* __restrict__ onrm, uint32_t* __restrict__ orgb) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int b = static_cast<int>(starts[s]);
  const uint32_t k = keys[b];
  const uint32_t i0 = vals[b];
  float4 p = xyz[i0], q = nrm[i0];
  uint32_t c = rgb[i0];
  float ax = p.x, ay = p.y, az = p.z, nx = q.x, ny = q.y, nz = q.z, cu = q.w;
  float cr = static_cast<float>((c >> 16) & 255u), cg = static_cast<float>((c >> 8) & 255u),
        cb = static_cast<float>(c & 255u);
  int e = b + 1;
  for (; e < n && keys[e] == k; ++e) {
    const uint32_t i = vals[e];
    p = xyz[i];
    q = nrm[i];
    c = rgb[i];
    ax = __fadd_rn(ax, p.x); ay = __fadd_rn(ay, p.y); az = __fadd_rn(az, p.z);
    nx = __fadd_rn(nx, q.x); ny = __fadd_rn(ny, q.y); nz = __fadd_rn(nz, q.z); cu = __fadd_rn(cu, q.w);
    cr = __fadd_rn(cr, static_cast<float>((c >> 16) & 255u));
    cg = __fadd_rn(cg, static_cast<float>((c >> 8) & 255u));
    cb = __fadd_rn(cb, static_cast<float>(c & 255u));
  }
  const float cnt = static_cast<float>(e - b);
  oxyz[s] = make_float4(__fdiv_rn(ax, cnt), __fdiv_rn(ay, cnt), __fdiv_rn(az, cnt), 0.f);
  onrm[s] = make_float4(__fdiv_rn(nx, cnt), __fdiv_rn(ny, cnt), __fdiv_rn(nz, cnt), __fdiv_rn(cu, cnt));
  const uint32_t r8 = static_cast<uint32_t>(static_cast<int>(__fdiv_rn(cr, cnt))) & 255u;
  const uint32_t g8 = static_cast<uint32_t>(static_cast<int>(__fdiv_rn(cg, cnt))) & 255u;
  const uint32_t b8 = static_cast<uint32_t>(static_cast<int>(__fdiv_rn(cb, cnt))) & 255u;
  orgb[s] = b8 | (g8 << 8) | (r8 << 16);
}

}  // namespace

lcr_cloud* concat_clouds(lcr_ctx* ctx, const lcr_cloud* a, const lcr_cloud* b);

lcr_cloud* voxel_run(lcr_ctx* ctx, const lcr_cloud* in, float lx, float ly, float lz) {
  if (!(lx > 0 && ly > 0 && lz > 0)) LCR_THROW(LCR_ERR_INVALID_ARG, "leaf size must be positive");
  const int n = static_cast<int>(in->n);
  if (n == 0) return cloud_alloc(ctx, 0);
  float4* box = static_cast<float4*>(dev_alloc(ctx, 2 * sizeof(float4) + sizeof(VoxelSetup)));
  VoxelSetup* vs = reinterpret_cast<VoxelSetup*>(box + 2);
  bbox(ctx, in->xyz, n, box);
  LCR_LAUNCH(ctx, k_voxel_setup, 1, 32, 0, box, lx, ly, lz, vs);
  uint32_t* keys = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * n));
  uint32_t* vals = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * n));
  uint8_t* flags = static_cast<uint8_t*>(dev_alloc(ctx, n));
  uint32_t* starts = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * n));
  LCR_LAUNCH(ctx, k_voxel_keys, (n + 255) / 256, 256, 0, in->xyz, n, vs, keys, vals);
  radix_sort_pairs(ctx, keys, vals, n, 32);
  LCR_LAUNCH(ctx, k_segment_heads, (n + 255) / 256, 256, 0, keys, n, flags);
  VoxelSetup* hv = static_cast<VoxelSetup*>(pinned(ctx, sizeof(VoxelSetup) + 64));
  const int nseg = compact_flags(ctx, flags, n, starts);  // synchronises
  CUDA_TRY(cudaMemcpyAsync(hv, vs, sizeof(VoxelSetup), cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  lcr_cloud* out = nullptr;
  if (hv->overflow) {
    lcr_cloud empty;
    out = concat_clouds(ctx, in, &empty);
  } else {
    out = cloud_alloc(ctx, nseg);
    if (nseg > 0)
      LCR_LAUNCH(ctx, k_voxel_centroids, (nseg + 127) / 128, 128, 0, keys, vals, n, starts, nseg, in->xyz, in->nrm,
                 in->rgb, out->xyz, out->nrm, out->rgb);
  }
  dev_free(ctx, box);
  dev_free(ctx, keys);
  dev_free(ctx, vals);
  dev_free(ctx, flags);
  dev_free(ctx, starts);
  return out;
}
