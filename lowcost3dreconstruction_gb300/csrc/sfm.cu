// Filters of the structure-from-motion branch (scripts/sfm.sh:82-85):
//  * CropBox around the centroid         pcl_tools/crop_cloud.cpp:81-97
//  * Euclidean cluster extraction        pcl_tools/cluster_extraction.cpp:90-130
//  * RANSAC plane segmentation           pcl_tools/planar_segmentation.cpp:80-110
// on the same search index and compaction primitives as the alignment path.
#include <algorithm>
#include <cmath>
#include <vector>

#include "lcr_internal.cuh"
#include "search.cuh"

namespace {

// ------------------------------------------------------------------ crop
// pcl::CropBox (identity transform): a finite point is inside when
// min <= p <= max on every axis; non-finite points are in neither output.
__global__ void k_box_flags(const float4* __restrict__ xyz, size_t n, float3 lo, float3 hi,
                            uint8_t* __restrict__ inside, uint8_t* __restrict__ outside) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i];
  const bool fin = finite3(p.x, p.y, p.z);
  const bool in = fin && p.x >= lo.x && p.y >= lo.y && p.z >= lo.z && p.x <= hi.x && p.y <= hi.y && p.z <= hi.z;
  inside[i] = in ? 1 : 0;
  outside[i] = fin && !in ? 1 : 0;
}

// ---------------------------------------------------------------- clusters
// Lock-free union-find over point indices with parent[v] <= v: a root is the
// smallest index of its component, so the final labels do not depend on the
// order in which the unions ran.
__device__ __forceinline__ uint32_t uf_find(volatile uint32_t* parent, uint32_t x) {
  uint32_t cur = parent[x];
  if (cur == x) return x;
  uint32_t prev = x, next;
  while (cur > (next = parent[cur])) {  // pointer jumping on the way up
    parent[prev] = next;
    prev = cur;
    cur = next;
  }
  return cur;
}

__device__ __forceinline__ void uf_unite(uint32_t* parent, uint32_t a, uint32_t b) {
  volatile uint32_t* vp = parent;
  uint32_t ra = uf_find(vp, a), rb = uf_find(vp, b);
  while (ra != rb) {
    if (ra > rb) {
      const uint32_t t = ra;
      ra = rb;
      rb = t;
    }
    const uint32_t old = atomicCAS(parent + rb, rb, ra);  // hook the larger root under the smaller
    if (old == rb) return;
    rb = uf_find(vp, old);
    ra = uf_find(vp, ra);
  }
}

// Radius visitor: unites the query with every point strictly closer than
// sqrt(r2) (FLANN's radius search keeps d < r^2, on the FP32 L2 distance).
struct RadiusUnion {
  float qx, qy, qz;
  bool qv;
  uint32_t qi;
  float r2;
  float4 tlo, thi;
  uint32_t* parent;
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return box_box_dist2(tlo, thi, lo, hi);
  }
  __device__ __forceinline__ bool still(float m) const { return m < r2; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) < r2;
  }
  __device__ __forceinline__ void scan(const float4* st) {
    for (int j = 0; j < 32; ++j) {
      const float4 p = st[j];
      const float d = exact_dist2(qx, qy, qz, p.x, p.y, p.z);
      if (!(d < r2)) continue;
      const uint32_t pi = __float_as_uint(p.w);
      if (pi > qi) uf_unite(parent, qi, pi);
    }
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() {}
};

__global__ void k_uf_init(uint32_t* __restrict__ parent, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) parent[i] = static_cast<uint32_t>(i);
}

__global__ void k_cluster_union(IndexView ix, float r2, uint32_t* parent) {
  __shared__ WarpScratch wss[8];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * (blockDim.x >> 5) + wib;
  if (tile >= ix.nleaf) return;
  const float4 p = ix.pts[static_cast<size_t>(tile) * 32 + lane];
  const bool qv = finite3(p.x, p.y, p.z);
  float4 tlo, thi;
  if (!tile_box(p.x, p.y, p.z, qv, tlo, thi)) return;
  RadiusUnion v;
  v.qx = p.x;
  v.qy = p.y;
  v.qz = p.z;
  v.qv = qv;
  v.qi = qv ? __float_as_uint(p.w) : 0u;
  v.r2 = r2;
  v.tlo = tlo;
  v.thi = thi;
  v.parent = parent;
  tile_traverse(ix, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), wss[wib]);
}

// label[i] = root of i; size[root] counts the finite members.
__global__ void k_uf_flatten(const float4* __restrict__ xyz, int n, uint32_t* parent, uint32_t* __restrict__ label,
                             unsigned int* __restrict__ size) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t r = uf_find(parent, static_cast<uint32_t>(i));
  label[i] = r;
  const float4 p = xyz[i];
  if (finite3(p.x, p.y, p.z)) atomicAdd(size + r, 1u);
}

__global__ void k_root_flags(const uint32_t* __restrict__ label, const unsigned int* __restrict__ size, int n,
                             unsigned int lo, unsigned int hi, uint8_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned int s = size[i];
  flags[i] = label[i] == static_cast<uint32_t>(i) && s >= lo && s <= hi && s > 0 ? 1 : 0;
}

__global__ void k_scatter_rank(const uint32_t* __restrict__ roots, int k, uint32_t* __restrict__ rank_of) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) rank_of[roots[j]] = static_cast<uint32_t>(j);
}

// key = rank of the point's cluster (k for points in no kept cluster), val = index.
__global__ void k_cluster_keys(const float4* __restrict__ xyz, const uint32_t* __restrict__ label,
                               const uint32_t* __restrict__ rank_of, int n, uint32_t k, uint32_t* __restrict__ keys,
                               uint32_t* __restrict__ vals, uint8_t* __restrict__ rest, int32_t* __restrict__ out_label) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i];
  uint32_t r = k;
  if (finite3(p.x, p.y, p.z)) r = min(rank_of[label[i]], k);
  keys[i] = r;
  vals[i] = static_cast<uint32_t>(i);
  rest[i] = r == k ? 1 : 0;
  out_label[i] = r == k ? -1 : static_cast<int32_t>(r);
}

// ------------------------------------------------------------------ plane
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__global__ void k_fin_flags(const float4* __restrict__ xyz, int n, uint8_t* __restrict__ f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float4 p = xyz[i];
    f[i] = finite3(p.x, p.y, p.z) ? 1 : 0;
  }
}

// Plane through three points of a sample, IEEE operations in a fixed order:
// n = (p1 - p0) x (p2 - p0), normalised; d = -(n . p0).  A sample whose
// cross product vanishes (repeated or collinear points) gives n = 0: no inliers.
__device__ float4 plane_of(float4 p0, float4 p1, float4 p2) {
  const float ax = __fsub_rn(p1.x, p0.x), ay = __fsub_rn(p1.y, p0.y), az = __fsub_rn(p1.z, p0.z);
  const float bx = __fsub_rn(p2.x, p0.x), by = __fsub_rn(p2.y, p0.y), bz = __fsub_rn(p2.z, p0.z);
  float nx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
  float ny = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
  float nz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
  const float nn = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
  if (!(nn > 0.f) || !(nn < LCR_INF)) return make_float4(0.f, 0.f, 0.f, LCR_INF);
  const float len = __fsqrt_rn(nn);
  nx = __fdiv_rn(nx, len);
  ny = __fdiv_rn(ny, len);
  nz = __fdiv_rn(nz, len);
  const float d = -__fadd_rn(__fadd_rn(__fmul_rn(nx, p0.x), __fmul_rn(ny, p0.y)), __fmul_rn(nz, p0.z));
  return make_float4(nx, ny, nz, d);
}

// |n . p + d| in a fixed order: ((nx x + ny y) + nz z) + d.
__device__ __forceinline__ float plane_dist(const float4 c, const float4 p) {
  return fabsf(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.x, p.x), __fmul_rn(c.y, p.y)), __fmul_rn(c.z, p.z)), c.w));
}

// Hypothesis h samples finite points fin[hash(seed, h, j) % nf], j = 0, 1, 2.
__global__ void k_plane_hyp(const float4* __restrict__ xyz, const uint32_t* __restrict__ fin, int nf, int H,
                            uint64_t seed, float4* __restrict__ coef) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= H) return;
  float4 p[3];
  for (int j = 0; j < 3; ++j) {
    const uint64_t r = mix64(seed ^ (static_cast<uint64_t>(h) << 2) ^ static_cast<uint64_t>(j));
    p[j] = xyz[fin[r % static_cast<uint64_t>(nf)]];
  }
  coef[h] = plane_of(p[0], p[1], p[2]);
}

// count[h] = number of finite points with |n_h . p + d_h| < t.  A block holds
// 32 hypotheses in shared memory and a chunk of points.
constexpr int kHypPerBlock = 32;
__global__ void __launch_bounds__(256) k_plane_count(const float4* __restrict__ xyz, int n,
                                                     const float4* __restrict__ coef, int H, float t,
                                                     unsigned int* __restrict__ count) {
  __shared__ float4 cs[kHypPerBlock];
  __shared__ unsigned int acc[kHypPerBlock];
  const int h0 = blockIdx.y * kHypPerBlock;
  if (threadIdx.x < kHypPerBlock) {
    cs[threadIdx.x] = h0 + threadIdx.x < H ? coef[h0 + threadIdx.x] : make_float4(0.f, 0.f, 0.f, LCR_INF);
    acc[threadIdx.x] = 0u;
  }
  __syncthreads();
  unsigned int c[kHypPerBlock];
#pragma unroll
  for (int h = 0; h < kHypPerBlock; ++h) c[h] = 0u;
  const int per = 4096;
  const int i0 = blockIdx.x * per, i1 = min(n, i0 + per);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const float4 p = xyz[i];
    if (!finite3(p.x, p.y, p.z)) continue;
#pragma unroll
    for (int h = 0; h < kHypPerBlock; ++h) c[h] += plane_dist(cs[h], p) < t ? 1u : 0u;
  }
#pragma unroll
  for (int h = 0; h < kHypPerBlock; ++h) {
    unsigned int v = c[h];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(LCR_FULL, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&acc[h], v);
  }
  __syncthreads();
  if (threadIdx.x < kHypPerBlock && acc[threadIdx.x] && h0 + threadIdx.x < H)
    atomicAdd(&count[h0 + threadIdx.x], acc[threadIdx.x]);
}

// Smallest-eigenvalue eigenvector of a symmetric 3x3 (FP64, cyclic Jacobi).
__device__ void jacobi_smallest(double a[3][3], double v_out[3]) {
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int sweep = 0; sweep < 16; ++sweep) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    if (off == 0.0) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(tt * tt + 1.0), s = tt * c;
        for (int k = 0; k < 3; ++k) {  // A <- J^T A J
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
  int m = 0;
  if (a[1][1] < a[m][m]) m = 1;
  if (a[2][2] < a[m][m]) m = 2;
  for (int k = 0; k < 3; ++k) v_out[k] = v[k][m];
}

// One block: the best hypothesis (most inliers, then the lowest index), the
// FP64 mean and covariance of its inliers (per-thread strided sums, then a
// fixed tree), and the least-squares plane through them: normal = eigenvector
// of the smallest eigenvalue (sign: that of the hypothesis), d = -n . mean.
__global__ void __launch_bounds__(256) k_plane_refine(const float4* __restrict__ xyz, int n,
                                                      const float4* __restrict__ coef,
                                                      const unsigned int* __restrict__ count, int H, float t,
                                                      float4* __restrict__ out, unsigned int* __restrict__ best_count) {
  __shared__ unsigned long long bk[256];
  __shared__ double red[10][256];
  const int tid = threadIdx.x;
  unsigned long long k = 0ull;
  for (int h = tid; h < H; h += 256) {
    const unsigned long long key = (static_cast<unsigned long long>(count[h]) << 32) | (0xffffffffu - h);
    k = key > k ? key : k;
  }
  bk[tid] = k;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (tid < s && bk[tid + s] > bk[tid]) bk[tid] = bk[tid + s];
    __syncthreads();
  }
  const int best = static_cast<int>(0xffffffffu - static_cast<uint32_t>(bk[0] & 0xffffffffu));
  const float4 c = coef[best];
  double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // count, sx, sy, sz, sxx, sxy, sxz, syy, syz, szz
  for (int i = tid; i < n; i += 256) {
    const float4 p = xyz[i];
    if (!finite3(p.x, p.y, p.z) || !(plane_dist(c, p) < t)) continue;
    const double x = p.x, y = p.y, z = p.z;
    acc[0] += 1.0;
    acc[1] += x;
    acc[2] += y;
    acc[3] += z;
    acc[4] += x * x;
    acc[5] += x * y;
    acc[6] += x * z;
    acc[7] += y * y;
    acc[8] += y * z;
    acc[9] += z * z;
  }
  for (int j = 0; j < 10; ++j) red[j][tid] = acc[j];
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (tid < s)
      for (int j = 0; j < 10; ++j) red[j][tid] += red[j][tid + s];
    __syncthreads();
  }
  if (tid == 0) {
    const double m = red[0][0];
    *best_count = static_cast<unsigned int>(bk[0] >> 32);
    if (m < 3.0) {
      *out = c;
      return;
    }
    const double mx = red[1][0] / m, my = red[2][0] / m, mz = red[3][0] / m;
    double cov[3][3];
    cov[0][0] = red[4][0] / m - mx * mx;
    cov[0][1] = cov[1][0] = red[5][0] / m - mx * my;
    cov[0][2] = cov[2][0] = red[6][0] / m - mx * mz;
    cov[1][1] = red[7][0] / m - my * my;
    cov[1][2] = cov[2][1] = red[8][0] / m - my * mz;
    cov[2][2] = red[9][0] / m - mz * mz;
    double nv[3];
    jacobi_smallest(cov, nv);
    if (nv[0] * c.x + nv[1] * c.y + nv[2] * c.z < 0.0)
      for (double& e : nv) e = -e;
    const double d = -(nv[0] * mx + nv[1] * my + nv[2] * mz);
    *out = make_float4(static_cast<float>(nv[0]), static_cast<float>(nv[1]), static_cast<float>(nv[2]),
                       static_cast<float>(d));
  }
}

__global__ void k_plane_flags(const float4* __restrict__ xyz, int n, const float4* __restrict__ coef, float t,
                              uint8_t* __restrict__ in, uint8_t* __restrict__ rest) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i];
  const bool on = finite3(p.x, p.y, p.z) && plane_dist(*coef, p) < t;
  in[i] = on ? 1 : 0;
  rest[i] = on ? 0 : 1;
}

}  // namespace

void plane_segment_run(lcr_ctx* ctx, const lcr_cloud* in, double threshold, int hypotheses, uint64_t seed,
                       float coefficients[4], size_t* ninliers, lcr_cloud** plane, lcr_cloud** rest) {
  const int n = static_cast<int>(in->n);
  const int H = hypotheses;
  const float t = static_cast<float>(threshold);
  const size_t b4 = 4 * static_cast<size_t>(n) + 16;
  char* blk = static_cast<char*>(dev_alloc(ctx, 2 * b4 + 2 * static_cast<size_t>(n) + 32 * static_cast<size_t>(H) + 256));
  uint32_t* fin = reinterpret_cast<uint32_t*>(blk);
  uint32_t* idx = reinterpret_cast<uint32_t*>(blk + b4);
  uint8_t* f0 = reinterpret_cast<uint8_t*>(blk + 2 * b4);
  uint8_t* f1 = f0 + n;
  float4* coef = reinterpret_cast<float4*>(blk + ((2 * b4 + 2 * static_cast<size_t>(n) + 15) & ~static_cast<size_t>(15)));
  unsigned int* count = reinterpret_cast<unsigned int*>(coef + H);
  float4* best = reinterpret_cast<float4*>(count + ((H + 3) & ~3));
  unsigned int* bestn = reinterpret_cast<unsigned int*>(best + 1);
  int nf = 0;
  if (n) {
    LCR_LAUNCH(ctx, k_fin_flags, (n + 255) / 256, 256, 0, in->xyz, n, f0);
    nf = compact_flags(ctx, f0, n, fin);
  }
  float4 hc = make_float4(0.f, 0.f, 0.f, 0.f);
  unsigned int hn = 0;
  if (nf >= 3) {
    CUDA_TRY(cudaMemsetAsync(count, 0, 4ull * H, ctx->stream));
    LCR_LAUNCH(ctx, k_plane_hyp, (H + 127) / 128, 128, 0, in->xyz, fin, nf, H, seed, coef);
    const dim3 grid((n + 4095) / 4096, (H + kHypPerBlock - 1) / kHypPerBlock);
    LCR_LAUNCH(ctx, k_plane_count, grid, 256, 0, in->xyz, n, coef, H, t, count);
    LCR_LAUNCH(ctx, k_plane_refine, 1, 256, 0, in->xyz, n, coef, count, H, t, best, bestn);
    CUDA_TRY(cudaMemcpyAsync(&hc, best, sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(&hn, bestn, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
  }
  int m_in = 0;
  if (n && hn > 0) {
    LCR_LAUNCH(ctx, k_plane_flags, (n + 255) / 256, 256, 0, in->xyz, n, best, t, f0, f1);
  } else if (n) {
    CUDA_TRY(cudaMemsetAsync(f0, 0, n, ctx->stream));
    CUDA_TRY(cudaMemsetAsync(f1, 1, n, ctx->stream));
  }
  if (n) m_in = compact_flags(ctx, f0, n, idx);
  coefficients[0] = hc.x;
  coefficients[1] = hc.y;
  coefficients[2] = hc.z;
  coefficients[3] = hc.w;
  *ninliers = static_cast<size_t>(hn > 0 ? m_in : 0);
  if (plane) {
    lcr_cloud* c = cloud_alloc(ctx, m_in);
    gather_cloud(ctx, in, idx, m_in, c);
    *plane = c;
  }
  if (rest) {
    const int m = n ? compact_flags(ctx, f1, n, idx) : 0;
    lcr_cloud* c = cloud_alloc(ctx, m);
    gather_cloud(ctx, in, idx, m, c);
    *rest = c;
  }
  sync(ctx);
  dev_free(ctx, blk);
}

void crop_box_run(lcr_ctx* ctx, const lcr_cloud* in, const float lo[3], const float hi[3], lcr_cloud** inside,
                  lcr_cloud** outside) {
  const size_t n = in->n;
  uint8_t* flags = static_cast<uint8_t*>(dev_alloc(ctx, 2 * n + 16));
  uint32_t* idx = static_cast<uint32_t*>(dev_alloc(ctx, 4 * n + 16));
  if (n)
    LCR_LAUNCH(ctx, k_box_flags, static_cast<unsigned>((n + 255) / 256), 256, 0, in->xyz, n,
               make_float3(lo[0], lo[1], lo[2]), make_float3(hi[0], hi[1], hi[2]), flags, flags + n);
  for (int side = 0; side < 2; ++side) {
    lcr_cloud** out = side == 0 ? inside : outside;
    if (!out) continue;
    const int m = n ? compact_flags(ctx, flags + side * n, static_cast<int>(n), idx) : 0;
    lcr_cloud* c = cloud_alloc(ctx, m);
    gather_cloud(ctx, in, idx, m, c);
    *out = c;
  }
  dev_free(ctx, flags);
  dev_free(ctx, idx);
  sync(ctx);
}

void euclidean_clusters_run(lcr_ctx* ctx, const lcr_cloud* in, double tolerance, size_t min_size, size_t max_size,
                            int32_t* host_labels, size_t* nclusters, lcr_cloud** clustered, lcr_cloud** rest) {
  const int n = static_cast<int>(in->n);
  *nclusters = 0;
  const size_t b4 = 4 * static_cast<size_t>(n) + 16;
  char* blk = static_cast<char*>(dev_alloc(ctx, 7 * b4 + 2 * static_cast<size_t>(n) + 64));
  uint32_t* parent = reinterpret_cast<uint32_t*>(blk);
  uint32_t* label = reinterpret_cast<uint32_t*>(blk + b4);
  unsigned int* size = reinterpret_cast<unsigned int*>(blk + 2 * b4);
  uint32_t* rank_of = reinterpret_cast<uint32_t*>(blk + 3 * b4);
  uint32_t* keys = reinterpret_cast<uint32_t*>(blk + 4 * b4);
  uint32_t* vals = reinterpret_cast<uint32_t*>(blk + 5 * b4);
  int32_t* dlabel = reinterpret_cast<int32_t*>(blk + 6 * b4);
  uint8_t* flags = reinterpret_cast<uint8_t*>(blk + 7 * b4);
  uint8_t* restf = flags + n;
  int k = 0;
  std::vector<uint32_t> roots;
  if (n > 0) {
    const IndexView ix = cloud_index(ctx, in).v;
    const float r2 = static_cast<float>(tolerance * tolerance);
    CUDA_TRY(cudaMemsetAsync(size, 0, b4, ctx->stream));
    CUDA_TRY(cudaMemsetAsync(rank_of, 0xff, b4, ctx->stream));  // roots of dropped clusters: no rank
    LCR_LAUNCH(ctx, k_uf_init, (n + 255) / 256, 256, 0, parent, n);
    LCR_LAUNCH(ctx, k_cluster_union, (ix.nleaf + 7) / 8, 256, 0, ix, r2, parent);
    LCR_LAUNCH(ctx, k_uf_flatten, (n + 255) / 256, 256, 0, in->xyz, n, parent, label, size);
    const unsigned int lo = static_cast<unsigned int>(std::min<size_t>(min_size, 0xffffffffu));
    const unsigned int hi = static_cast<unsigned int>(std::min<size_t>(max_size, 0xffffffffu));
    LCR_LAUNCH(ctx, k_root_flags, (n + 255) / 256, 256, 0, label, size, n, lo, hi, flags);
    k = compact_flags(ctx, flags, n, keys);  // kept roots, ascending
    // order the kept clusters: size descending, then smallest index first
    roots.resize(k);
    std::vector<unsigned int> sizes(k);
    if (k) {
      CUDA_TRY(cudaMemcpyAsync(roots.data(), keys, 4ull * k, cudaMemcpyDeviceToHost, ctx->stream));
      std::vector<unsigned int> all(n);
      CUDA_TRY(cudaMemcpyAsync(all.data(), size, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream));
      sync(ctx);
      for (int j = 0; j < k; ++j) sizes[j] = all[roots[j]];
      std::vector<int> order(k);
      for (int j = 0; j < k; ++j) order[j] = j;
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sizes[a] > sizes[b]; });
      std::vector<uint32_t> sorted(k);
      for (int j = 0; j < k; ++j) sorted[j] = roots[order[j]];
      roots.swap(sorted);
      CUDA_TRY(cudaMemcpyAsync(vals, roots.data(), 4ull * k, cudaMemcpyHostToDevice, ctx->stream));
      LCR_LAUNCH(ctx, k_scatter_rank, (k + 255) / 256, 256, 0, vals, k, rank_of);
      sync(ctx);  // the host vector feeding the copy goes out of scope below
    }
    LCR_LAUNCH(ctx, k_cluster_keys, (n + 255) / 256, 256, 0, in->xyz, label, rank_of, n, static_cast<uint32_t>(k),
               keys, vals, restf, dlabel);
  }
  *nclusters = static_cast<size_t>(k);
  if (host_labels && n) CUDA_TRY(cudaMemcpyAsync(host_labels, dlabel, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (clustered) {
    int m = 0;
    if (n) {
      int bits = 1;
      while ((1u << bits) <= static_cast<unsigned>(k)) ++bits;
      radix_sort_pairs(ctx, keys, vals, n, bits);  // stable: ascending index within a cluster
      m = n - compact_flags(ctx, restf, n, reinterpret_cast<uint32_t*>(parent));
    }
    lcr_cloud* c = cloud_alloc(ctx, m);
    gather_cloud(ctx, in, vals, m, c);
    *clustered = c;
  }
  if (rest) {
    const int m = n ? compact_flags(ctx, restf, n, reinterpret_cast<uint32_t*>(parent)) : 0;
    lcr_cloud* c = cloud_alloc(ctx, m);
    gather_cloud(ctx, in, reinterpret_cast<uint32_t*>(parent), m, c);
    *rest = c;
  }
  sync(ctx);
  dev_free(ctx, blk);
}
