// Exact k-nearest-neighbour queries (lcr_knn) and single ICP correspondence
// passes (lcr_correspondences), both on the warp-tile traversal.
#include <algorithm>
#include <cmath>

#include "search.cuh"

namespace {

__global__ void k_fill_knn(int32_t* __restrict__ idx, float* __restrict__ dist, size_t m) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < m) {
    idx[i] = -1;
    dist[i] = LCR_INF;
  }
}

// Queries are the Morton-sorted points of the query cloud's own index; results
// are scattered back to the query's original position.
__global__ void k_knn(IndexView ref, IndexView qry, int K, float cap, int self, int32_t* __restrict__ oidx,
                      float* __restrict__ odist) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t wbytes = K == 1 ? sizeof(WarpScratch) : knn_warp_bytes(K);
  unsigned char* wbase = smem + wib * wbytes;
  WarpScratch& ws = *reinterpret_cast<WarpScratch*>(wbase);
  const int tile = blockIdx.x * nw + wib;
  if (tile >= qry.nleaf) return;
  const float4 q = qry.pts[static_cast<size_t>(tile) * 32 + lane];
  const bool qv = finite3(q.x, q.y, q.z);
  float4 tlo, thi;
  if (!tile_box(q.x, q.y, q.z, qv, tlo, thi)) return;
  const uint32_t orig = __float_as_uint(q.w);
  if (K == 1) {
    NN1 v;
    tile_nn1(ref, q.x, q.y, q.z, qv, cap, tlo, thi, ws, v);
    if (qv && v.found()) {
      oidx[orig] = static_cast<int32_t>(key_idx(v.best));
      odist[orig] = key_dist(v.best);
    }
  } else {
    unsigned char* region = wbase + sizeof(KnnWarp);
    const unsigned long long* list = reinterpret_cast<const unsigned long long*>(region);
    tile_knn(ref, q.x, q.y, q.z, qv, K, cap, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), region,
             self ? tile : -1);
    if (qv) {
      for (int j = 0; j < K; ++j) {
        const unsigned long long k = list[j * 32 + lane];
        if (key_idx(k) == 0xffffffffu) break;
        oidx[static_cast<size_t>(orig) * K + j] = static_cast<int32_t>(key_idx(k));
        odist[static_cast<size_t>(orig) * K + j] = key_dist(k);
      }
    }
  }
}

// One correspondence pass: query = source point transformed by T (FP32).
__global__ void k_corr(IndexView tgt, IndexView src, Xf T, float cap, int32_t* __restrict__ oidx,
                       float* __restrict__ odist) {
  __shared__ WarpScratch wss[8];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * (blockDim.x >> 5) + wib;
  if (tile >= src.nleaf) return;
  const float4 p = src.pts[static_cast<size_t>(tile) * 32 + lane];
  const bool qv = finite3(p.x, p.y, p.z);
  float3 q = make_float3(0.f, 0.f, 0.f);
  if (qv) q = xf_apply(T, p.x, p.y, p.z);
  float4 tlo, thi;
  if (!tile_box(q.x, q.y, q.z, qv, tlo, thi)) return;
  NN1 v;
  tile_nn1(tgt, q.x, q.y, q.z, qv, cap, tlo, thi, wss[wib], v);
  if (qv && v.found()) {
    const uint32_t orig = __float_as_uint(p.w);
    oidx[orig] = static_cast<int32_t>(key_idx(v.best));
    odist[orig] = key_dist(v.best);
  }
}

}  // namespace

// Largest float whose double value is <= v: the FP32 form of PCL's
// `distance > max_dist_sqr` rejection (a float distance compared in double).
float float_cap(double v) {
  if (!(v < 3.4028234663852886e38)) return LCR_INF_HOST;
  float f = static_cast<float>(v);
  if (static_cast<double>(f) > v) f = std::nextafter(f, 0.0f);
  return f;
}

void knn_run(lcr_ctx* ctx, const lcr_cloud* ref, const lcr_cloud* query, int k, float cap, int32_t* d_idx,
             float* d_dist) {
  const size_t m = query->n * static_cast<size_t>(k);
  if (m == 0) return;
  LCR_LAUNCH(ctx, k_fill_knn, static_cast<unsigned>((m + 255) / 256), 256, 0, d_idx, d_dist, m);
  if (ref->n == 0) return;
  const IndexView rv = cloud_index(ctx, ref).v;
  const IndexView qv = cloud_index(ctx, query).v;
  const int nw = k == 1 ? 8 : (k <= 64 ? 4 : 2);
  const size_t smem = nw * (k == 1 ? sizeof(WarpScratch) : knn_warp_bytes(k));
  if (smem > 227 * 1024) LCR_THROW(LCR_ERR_INVALID_ARG, "k=%d too large", k);
  CUDA_TRY(cudaFuncSetAttribute(k_knn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const int grid = (qv.nleaf + nw - 1) / nw;
  LCR_LAUNCH(ctx, k_knn, grid, nw * 32, smem, rv, qv, k, cap, ref == query ? 1 : 0, d_idx, d_dist);
}

void corr_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const double* T, double dmax, int32_t* d_idx,
              float* d_dist) {
  if (src->n == 0) return;
  LCR_LAUNCH(ctx, k_fill_knn, static_cast<unsigned>((src->n + 255) / 256), 256, 0, d_idx, d_dist, src->n);
  if (tgt->n == 0) return;
  const IndexView tv = cloud_index(ctx, tgt).v;
  const IndexView sv = cloud_index(ctx, src).v;
  Xf X;
  for (int i = 0; i < 12; ++i) X.m[i] = static_cast<float>(T[i]);
  const float cap = float_cap(dmax * dmax);
  LCR_LAUNCH(ctx, k_corr, (sv.nleaf + 7) / 8, 256, 0, tv, sv, X, cap, d_idx, d_dist);
}
