// Warp-cooperative exact search over a Morton-sorted leaf hierarchy.
//
// A warp owns a tile of 32 queries (one per lane; spatially coherent because
// queries are Morton-sorted too).  It walks the 32-ary box hierarchy of the
// reference cloud once for the whole tile: at an internal node each lane tests
// one child box against the tile (its box plus the largest per-lane search
// radius), the passing children are pushed nearest-first onto a warp-private
// stack in shared memory; at a leaf the 32 points are loaded with one coalesced
// float4 per lane, staged in shared memory, and every lane that can still
// improve (per-lane box test) scans all 32 staged points against its own query.
// Pruning uses strict lower bounds (see box_dist2) and '<=' comparisons, so the
// result is the exact k nearest under the (distance, index) order -- the
// lowest-index tie rule.
#pragma once

#include "lcr_internal.cuh"

#define LCR_INF __int_as_float(0x7f800000)

constexpr int kStack = 32 * kMaxLevels + 32;

struct WarpScratch {
  uint32_t node[kStack];
  float d[kStack];
  float4 stage[32];
};

// Visitor contract (per-lane state, warp-synchronous calls):
//   float metric(lo, hi)  warp-level pruning metric of a node (tile vs box)
//   bool  still(m)        node with metric m may still hold useful points
//   bool  need(lo, hi)    this lane needs the leaf
//   void  scan(stage)     this lane scans the 32 staged points
//   void  refresh()       recompute the warp-level radius after a scan
template <class V>
__device__ __forceinline__ void tile_traverse(const IndexView& ix, V& vis, float cx, float cy, float cz,
                                              WarpScratch& ws) {
  const int lane = threadIdx.x & 31;
  int sp = 1;
  if (lane == 0) {
    ws.node[0] = static_cast<uint32_t>(ix.top) << 27;
    ws.d[0] = 0.f;
  }
  __syncwarp();
  while (sp > 0) {
    --sp;
    const uint32_t node = ws.node[sp];
    const float nd = ws.d[sp];
    __syncwarp();
    if (!vis.still(nd)) continue;
    const int level = static_cast<int>(node >> 27);
    const int id = static_cast<int>(node & 0x07ffffffu);
    if (level == 0) {
      const float4 lo = ix.lo[0][id], hi = ix.hi[0][id];
      const bool need = vis.need(lo, hi);
      if (!__any_sync(LCR_FULL, need)) continue;
      ws.stage[lane] = ix.pts[static_cast<size_t>(id) * 32 + lane];
      __syncwarp();
      if (need) vis.scan(ws.stage);
      __syncwarp();
      vis.refresh();
    } else {
      const int cl = level - 1;
      const int c = id * 32 + lane;
      const bool has = c < ix.count[cl];
      float m = LCR_INF, dord = LCR_INF;
      if (has) {
        const float4 lo = ix.lo[cl][c], hi = ix.hi[cl][c];
        m = vis.metric(lo, hi);
        dord = box_dist2(lo, hi, cx, cy, cz);
      }
      const bool pass = has && vis.still(m);
      const unsigned mask = __ballot_sync(LCR_FULL, pass);
      // Position among the passing children: farther children sit deeper in the
      // stack so the nearest is popped first.
      int pos = 0;
#pragma unroll 4
      for (int j = 0; j < 32; ++j) {
        const float dj = __shfl_sync(LCR_FULL, dord, j);
        if (((mask >> j) & 1u) && (dj > dord || (dj == dord && j > lane))) ++pos;
      }
      if (pass) {
        ws.node[sp + pos] = (static_cast<uint32_t>(cl) << 27) | static_cast<uint32_t>(c);
        ws.d[sp + pos] = m;
      }
      sp += __popc(mask);
      __syncwarp();
    }
  }
}

// Tile box of the valid queries of a warp.  Returns false if none is valid.
__device__ __forceinline__ bool tile_box(float x, float y, float z, bool v, float4& lo, float4& hi) {
  lo.x = warp_min(v ? x : LCR_INF);
  lo.y = warp_min(v ? y : LCR_INF);
  lo.z = warp_min(v ? z : LCR_INF);
  hi.x = warp_max(v ? x : -LCR_INF);
  hi.y = warp_max(v ? y : -LCR_INF);
  hi.z = warp_max(v ? z : -LCR_INF);
  lo.w = hi.w = 0.f;
  return __any_sync(LCR_FULL, v);
}

// ------------------------------------------------------------ 1-NN visitor
// best starts at (cap, 0xffffffff): a point is accepted iff its distance <= cap.
struct NN1 {
  float qx, qy, qz;
  bool qv;
  unsigned long long best;
  float4 bp;
  float4 tlo, thi;
  float R;

  __device__ __forceinline__ void init(float x, float y, float z, bool v, float cap, const float4& lo,
                                       const float4& hi) {
    qx = x; qy = y; qz = z; qv = v;
    best = make_key(cap, 0xffffffffu);
    bp = make_float4(0.f, 0.f, 0.f, 0.f);
    tlo = lo; thi = hi;
    refresh();
  }
  __device__ __forceinline__ float bound() const { return key_dist(best); }
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return box_box_dist2(lo, hi, tlo, thi);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) <= bound();
  }
  __device__ __forceinline__ void scan(const float4* st) {
#pragma unroll 8
    for (int j = 0; j < 32; ++j) {
      const float4 p = st[j];
      const float d = exact_dist2(qx, qy, qz, p.x, p.y, p.z);
      const unsigned long long k = make_key(d, __float_as_uint(p.w));
      if (k < best) {
        best = k;
        bp = p;
      }
    }
  }
  __device__ __forceinline__ void refresh() { R = warp_max(qv ? bound() : -LCR_INF); }
  __device__ __forceinline__ bool found() const { return key_idx(best) != 0xffffffffu; }
};

// ---------------------------------------------------------- k-NN visitor
// Sorted per-lane list of K keys in shared memory, column layout list[j*32+lane]
// (conflict-free whatever position each lane touches).
struct NNK {
  float qx, qy, qz;
  bool qv;
  int K;
  unsigned long long* list;
  float4 tlo, thi;
  float R;
  int lane;

  __device__ __forceinline__ void init(float x, float y, float z, bool v, float cap, int k, unsigned long long* l,
                                       const float4& lo, const float4& hi) {
    qx = x; qy = y; qz = z; qv = v; K = k; list = l;
    lane = threadIdx.x & 31;
    const unsigned long long e = make_key(cap, 0xffffffffu);
    for (int j = 0; j < K; ++j) list[j * 32 + lane] = e;
    tlo = lo; thi = hi;
    __syncwarp();
    refresh();
  }
  __device__ __forceinline__ float bound() const { return key_dist(list[(K - 1) * 32 + lane]); }
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return box_box_dist2(lo, hi, tlo, thi);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) <= bound();
  }
  __device__ __forceinline__ void scan(const float4* st) {
    unsigned long long worst = list[(K - 1) * 32 + lane];
    for (int j = 0; j < 32; ++j) {
      const float4 p = st[j];
      const float d = exact_dist2(qx, qy, qz, p.x, p.y, p.z);
      const unsigned long long k = make_key(d, __float_as_uint(p.w));
      if (k < worst) {
        int pos = K - 1;
        while (pos > 0) {
          const unsigned long long prev = list[(pos - 1) * 32 + lane];
          if (prev <= k) break;
          list[pos * 32 + lane] = prev;
          --pos;
        }
        list[pos * 32 + lane] = k;
        worst = list[(K - 1) * 32 + lane];
      }
    }
  }
  __device__ __forceinline__ void refresh() { R = warp_max(qv ? bound() : -LCR_INF); }
};
