// Search-index build: bounding box -> 30-bit Hilbert keys of a uniform 1024^3
// grid over the cloud's cube -> stable radix sort (the sorted grid, i.e. the
// voxel hash in key order) -> points gathered in key order as float4 with the
// original index in w -> leaf boxes (32 points) -> 32-ary box levels.
#include <algorithm>

#include "lcr_internal.cuh"

namespace {

// 30-bit 3D Hilbert index of 10-bit grid coordinates (Skilling, "Programming
// the Hilbert curve", AIP Conf. Proc. 707, 2004: axes -> transposed index, then
// bit interleave).  Consecutive Hilbert cells are face neighbours, so runs of 32
// consecutive points form compact leaves -- about half the leaf visits of a
// Morton order on depth-camera surfaces.
__device__ __forceinline__ uint32_t hilbert10(uint32_t x0, uint32_t x1, uint32_t x2) {
  uint32_t X[3] = {x0, x1, x2};
#pragma unroll
  for (uint32_t Q = 1u << 9; Q > 1u; Q >>= 1) {
    const uint32_t P = Q - 1u;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  X[2] ^= X[1];
  uint32_t t = 0;
#pragma unroll
  for (uint32_t Q = 1u << 9; Q > 1u; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1u;
  X[0] ^= t;
  X[1] ^= t;
  X[2] ^= t;
  uint32_t h = 0;
#pragma unroll
  for (int b = 9; b >= 0; --b)
#pragma unroll
    for (int i = 0; i < 3; ++i) h = (h << 1) | ((X[i] >> b) & 1u);
  return h;
}

__global__ void k_curve_keys(const float4* __restrict__ xyz, int n, const float4* __restrict__ box,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = xyz[i];
  uint32_t key = 0xffffffffu;
  if (finite3(p.x, p.y, p.z)) {
    const float4 lo = box[0], hi = box[1];
    const float ext = fmaxf(fmaxf(hi.x - lo.x, hi.y - lo.y), hi.z - lo.z);
    const float s = ext > 0.f ? 1023.0f / ext : 0.f;
    const uint32_t ix = min(1023u, static_cast<uint32_t>(fmaxf((p.x - lo.x) * s, 0.f)));
    const uint32_t iy = min(1023u, static_cast<uint32_t>(fmaxf((p.y - lo.y) * s, 0.f)));
    const uint32_t iz = min(1023u, static_cast<uint32_t>(fmaxf((p.z - lo.z) * s, 0.f)));
    key = hilbert10(ix, iy, iz);
  }
  keys[i] = key;
  vals[i] = static_cast<uint32_t>(i);
}

__global__ void k_gather_sorted(const float4* __restrict__ xyz, const uint32_t* __restrict__ keys,
                                const uint32_t* __restrict__ vals, int n, int npad, float4* __restrict__ pts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npad) return;
  float4 o;
  if (i < n && keys[i] != 0xffffffffu) {
    const uint32_t s = vals[i];
    const float4 p = xyz[s];
    o = make_float4(p.x, p.y, p.z, __uint_as_float(s));
  } else {
    const float nan = __int_as_float(0x7fc00000);
    o = make_float4(nan, nan, nan, __uint_as_float(0xffffffffu));
  }
  pts[i] = o;
}

// One warp per leaf; sentinel (non-finite) slots do not extend the box.  A leaf
// with no finite point gets the empty box [+inf, -inf].
__global__ void k_leaf_boxes(const float4* __restrict__ pts, int nleaf, float4* __restrict__ lo,
                             float4* __restrict__ hi) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nleaf) return;
  const float4 p = pts[static_cast<size_t>(warp) * 32 + lane];
  const bool f = finite3(p.x, p.y, p.z);
  const float inf = __int_as_float(0x7f800000);
  const float lx = warp_min(f ? p.x : inf), ly = warp_min(f ? p.y : inf), lz = warp_min(f ? p.z : inf);
  const float hx = warp_max(f ? p.x : -inf), hy = warp_max(f ? p.y : -inf), hz = warp_max(f ? p.z : -inf);
  if (lane == 0) {
    lo[warp] = make_float4(lx, ly, lz, 0.f);
    hi[warp] = make_float4(hx, hy, hz, 0.f);
  }
}

__global__ void k_level_boxes(const float4* __restrict__ clo, const float4* __restrict__ chi, int nchild, int nnode,
                              float4* __restrict__ lo, float4* __restrict__ hi) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nnode) return;
  const int c = warp * 32 + lane;
  const float inf = __int_as_float(0x7f800000);
  float4 a = make_float4(inf, inf, inf, 0.f), b = make_float4(-inf, -inf, -inf, 0.f);
  if (c < nchild) {
    a = clo[c];
    b = chi[c];
  }
  const float lx = warp_min(a.x), ly = warp_min(a.y), lz = warp_min(a.z);
  const float hx = warp_max(b.x), hy = warp_max(b.y), hz = warp_max(b.z);
  if (lane == 0) {
    lo[warp] = make_float4(lx, ly, lz, 0.f);
    hi[warp] = make_float4(hx, hy, hz, 0.f);
  }
}

// Subset index: position of every kept input point among the kept points.
__global__ void k_rank_of_kept(const uint32_t* __restrict__ kept, int nkeep, uint32_t* __restrict__ rank) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nkeep) rank[kept[j]] = static_cast<uint32_t>(j);
}

// flags over the sorted slots of the source index: slot holds a kept point
__global__ void k_slot_kept(const float4* __restrict__ pts, int npad, const uint8_t* __restrict__ keep,
                            uint8_t* __restrict__ flags) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= npad) return;
  const uint32_t w = __float_as_uint(pts[s].w);
  flags[s] = (w != 0xffffffffu && keep[w]) ? 1 : 0;
}

__global__ void k_gather_subset(const float4* __restrict__ src, const uint32_t* __restrict__ slots, int nkeep,
                                const uint32_t* __restrict__ rank, int npad, float4* __restrict__ pts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npad) return;
  float4 o;
  if (i < nkeep) {
    const float4 p = src[slots[i]];
    o = make_float4(p.x, p.y, p.z, __uint_as_float(rank[__float_as_uint(p.w)]));
  } else {
    const float nan = __int_as_float(0x7fc00000);
    o = make_float4(nan, nan, nan, __uint_as_float(0xffffffffu));
  }
  pts[i] = o;
}

inline size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

}  // namespace

namespace {

// Allocates an index for n points (one block: sorted points, then lo/hi boxes
// of every level).
Index* index_alloc(lcr_ctx* ctx, int n) {
  if (n <= 0) LCR_THROW(LCR_ERR_EMPTY, "cannot index an empty cloud");
  int counts[kMaxLevels + 1];
  int levels = 0;
  counts[0] = (n + 31) / 32;
  while (counts[levels] > 1) {
    if (levels + 1 >= kMaxLevels) LCR_THROW(LCR_ERR_INVALID_ARG, "cloud too large for the index (%d points)", n);
    counts[levels + 1] = (counts[levels] + 31) / 32;
    ++levels;
  }
  Index* ix = new Index();
  IndexView& v = ix->v;
  v.n = n;
  v.nleaf = counts[0];
  v.top = levels;
  const size_t npad = static_cast<size_t>(v.nleaf) * 32;
  size_t bytes = align256(npad * sizeof(float4));
  for (int l = 0; l <= levels; ++l) bytes += 2 * align256(static_cast<size_t>(counts[l]) * sizeof(float4));
  char* blk = nullptr;
  try {
    blk = static_cast<char*>(dev_alloc(ctx, bytes));
  } catch (...) {
    delete ix;
    throw;
  }
  ix->block = blk;
  ix->bytes = bytes;
  size_t off = 0;
  v.pts = reinterpret_cast<float4*>(blk);
  off += align256(npad * sizeof(float4));
  for (int l = 0; l < kMaxLevels; ++l) {
    v.lo[l] = v.hi[l] = nullptr;
    v.count[l] = 0;
  }
  for (int l = 0; l <= levels; ++l) {
    v.count[l] = counts[l];
    v.lo[l] = reinterpret_cast<float4*>(blk + off);
    off += align256(static_cast<size_t>(counts[l]) * sizeof(float4));
    v.hi[l] = reinterpret_cast<float4*>(blk + off);
    off += align256(static_cast<size_t>(counts[l]) * sizeof(float4));
  }
  return ix;
}

// Leaf boxes and the box levels above them, from the sorted points.
void index_boxes(lcr_ctx* ctx, Index* ix) {
  IndexView& v = ix->v;
  LCR_LAUNCH(ctx, k_leaf_boxes, (v.nleaf * 32 + 255) / 256, 256, 0, v.pts, v.nleaf, const_cast<float4*>(v.lo[0]),
             const_cast<float4*>(v.hi[0]));
  for (int l = 1; l <= v.top; ++l) {
    LCR_LAUNCH(ctx, k_level_boxes, (v.count[l] * 32 + 255) / 256, 256, 0, v.lo[l - 1], v.hi[l - 1], v.count[l - 1],
               v.count[l], const_cast<float4*>(v.lo[l]), const_cast<float4*>(v.hi[l]));
  }
}

}  // namespace

Index* build_index(lcr_ctx* ctx, const float4* xyz, int n) {
  Index* ix = index_alloc(ctx, n);
  IndexView& v = ix->v;
  const size_t npad = static_cast<size_t>(v.nleaf) * 32;
  const size_t kv_bytes = align256(sizeof(uint32_t) * 2 * static_cast<size_t>(n));
  char* scratch = static_cast<char*>(dev_alloc(ctx, kv_bytes + 2 * sizeof(float4)));
  uint32_t* keys = reinterpret_cast<uint32_t*>(scratch);
  uint32_t* vals = keys + n;
  float4* box = reinterpret_cast<float4*>(scratch + kv_bytes);
  bbox(ctx, xyz, n, box);
  LCR_LAUNCH(ctx, k_curve_keys, (n + 255) / 256, 256, 0, xyz, n, box, keys, vals);
  radix_sort_pairs(ctx, keys, vals, n, 32);
  LCR_LAUNCH(ctx, k_gather_sorted, static_cast<int>((npad + 255) / 256), 256, 0, xyz, keys, vals, n,
             static_cast<int>(npad), const_cast<float4*>(v.pts));
  index_boxes(ctx, ix);
  dev_free(ctx, scratch);
  return ix;
}

// Index of the points of a cloud kept by keep[] (input order; `kept` lists
// them, nkeep of them), numbered by their position among the kept points --
// the numbering of the compacted cloud.  No new sort: the source's sorted
// order restricted to the kept points keeps its spatial coherence.
Index* subset_index(lcr_ctx* ctx, const Index& src, const uint8_t* keep, const uint32_t* kept, int nkeep) {
  Index* ix = index_alloc(ctx, nkeep);
  IndexView& v = ix->v;
  const int npad_src = src.v.nleaf * 32;
  const int npad = v.nleaf * 32;
  char* tmp = static_cast<char*>(dev_alloc(ctx, sizeof(uint32_t) * (static_cast<size_t>(src.v.n) + npad_src) +
                                                   static_cast<size_t>(npad_src) + 256));
  uint32_t* rank = reinterpret_cast<uint32_t*>(tmp);
  uint32_t* slots = rank + src.v.n;
  uint8_t* flags = reinterpret_cast<uint8_t*>(slots + npad_src);
  LCR_LAUNCH(ctx, k_rank_of_kept, (nkeep + 255) / 256, 256, 0, kept, nkeep, rank);
  LCR_LAUNCH(ctx, k_slot_kept, (npad_src + 255) / 256, 256, 0, src.v.pts, npad_src, keep, flags);
  compact_flags_async(ctx, flags, npad_src, slots);
  LCR_LAUNCH(ctx, k_gather_subset, (npad + 255) / 256, 256, 0, src.v.pts, slots, nkeep, rank, npad,
             const_cast<float4*>(v.pts));
  index_boxes(ctx, ix);
  dev_free(ctx, tmp);
  return ix;
}

Index* share_index(Index* ix) {
  if (ix) ++ix->refs;
  return ix;
}

void free_index(lcr_ctx* ctx, Index* ix) {
  if (!ix || --ix->refs > 0) return;
  dev_free(ctx, ix->block);
  delete ix;
}
