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

// Deepest stack: the root, then 31 more entries per level below it (a popped
// node pushes at most 32 children): 1 + 31 * top <= 156 for top <= 5.
constexpr int kStack = 32 * (kMaxLevels - 1) + 8;

// A leaf's 32 points by coordinate: one 16-byte shared load gives the same
// coordinate of four consecutive points, i.e. two ready pairs for the paired
// FP32 distance.
struct SoaStage {
  float x[32], y[32], z[32];
  uint32_t i[32];
};

struct WarpScratch {
  uint32_t node[kStack];
  float d[kStack];
  union {  // one layout per visitor (stages_soa)
    float4 stage[32];
    SoaStage soa;
  };
  // Four sub-tiles of 8 consecutive lanes (nearby along the Hilbert order):
  // their boxes and largest per-lane radii.  A node must come within the
  // radius of some sub-tile, so a tile whose 32 queries straddle two distant
  // surfaces does not admit everything between them.
  float4 sub_lo[4], sub_hi[4];
  float sub_r[4];
  uint8_t qown[32];  // compacted leaf scans: lane of the r-th lane that needs the leaf
};

__device__ __forceinline__ void subtile_setup(float x, float y, float z, bool v, WarpScratch& ws) {
  const float inf = __int_as_float(0x7f800000);
  float lx = v ? x : inf, ly = v ? y : inf, lz = v ? z : inf;
  float hx = v ? x : -inf, hy = v ? y : -inf, hz = v ? z : -inf;
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) {
    lx = fminf(lx, __shfl_xor_sync(LCR_FULL, lx, o));
    ly = fminf(ly, __shfl_xor_sync(LCR_FULL, ly, o));
    lz = fminf(lz, __shfl_xor_sync(LCR_FULL, lz, o));
    hx = fmaxf(hx, __shfl_xor_sync(LCR_FULL, hx, o));
    hy = fmaxf(hy, __shfl_xor_sync(LCR_FULL, hy, o));
    hz = fmaxf(hz, __shfl_xor_sync(LCR_FULL, hz, o));
  }
  const int lane = threadIdx.x & 31;
  if ((lane & 7) == 0) {
    ws.sub_lo[lane >> 3] = make_float4(lx, ly, lz, 0.f);
    ws.sub_hi[lane >> 3] = make_float4(hx, hy, hz, 0.f);
  }
  __syncwarp();
}

// Per-sub-tile largest bound (invalid lanes excluded); returns the tile maximum.
__device__ __forceinline__ float subtile_radius(float b, bool v, WarpScratch& ws) {
  float r = v ? b : -__int_as_float(0x7f800000);
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) r = fmaxf(r, __shfl_xor_sync(LCR_FULL, r, o));
  const int lane = threadIdx.x & 31;
  __syncwarp();
  if ((lane & 7) == 0) ws.sub_r[lane >> 3] = r;
  r = fmaxf(r, __shfl_xor_sync(LCR_FULL, r, 8));
  r = fmaxf(r, __shfl_xor_sync(LCR_FULL, r, 16));
  __syncwarp();
  return r;
}

// Smallest squared gap from the node box to a sub-tile whose radius reaches
// it; +inf when none does.
__device__ __forceinline__ float subtile_metric(const float4& lo, const float4& hi, const WarpScratch& ws) {
  float m = __int_as_float(0x7f800000);
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const float d = box_box_dist2(lo, hi, ws.sub_lo[g], ws.sub_hi[g]);
    if (d <= ws.sub_r[g]) m = fminf(m, d);
  }
  return m;
}

// A visitor that declares `static constexpr bool kSoa = true` receives the
// staged leaf as a SoaStage, every other one as float4[32].
template <class V, class = void>
struct stages_soa {
  static constexpr bool value = false;
};
template <class V>
struct stages_soa<V, decltype(void(V::kSoa))> {
  static constexpr bool value = V::kSoa;
};

// Stages leaf `id` of ix for the warp (each lane one point, coalesced).
template <bool Soa>
__device__ __forceinline__ void stage_leaf(const IndexView& ix, int id, WarpScratch& ws) {
  const int lane = threadIdx.x & 31;
  const float4 p = ix.pts[static_cast<size_t>(id) * 32 + lane];
  if constexpr (Soa) {
    ws.soa.x[lane] = p.x;
    ws.soa.y[lane] = p.y;
    ws.soa.z[lane] = p.z;
    ws.soa.i[lane] = __float_as_uint(p.w);
  } else {
    ws.stage[lane] = p;
  }
}

// A visitor with `static constexpr bool kWarpScan = true` scans a leaf with
// the whole warp (scan_warp(stage, need), called by every lane).
template <class V, class = void>
struct scans_warp {
  static constexpr bool value = false;
};
template <class V>
struct scans_warp<V, decltype(void(V::kWarpScan))> {
  static constexpr bool value = V::kWarpScan;
};

// Stages leaf `id` in the visitor's layout and lets the lanes that need it
// scan it (warp-uniform call).
template <class V>
__device__ __forceinline__ void scan_staged(const IndexView& ix, int id, bool need, V& vis, WarpScratch& ws) {
  constexpr bool soa = stages_soa<V>::value;
  stage_leaf<soa>(ix, id, ws);
  __syncwarp();
  if constexpr (scans_warp<V>::value) {
    vis.scan_warp(ws.soa, need);
  } else if (need) {
    if constexpr (soa) vis.scan(ws.soa);
    else vis.scan(ws.stage);
  }
  __syncwarp();
}

// The exact_dist2 of one query to staged points j .. j+3 (j a multiple of 4).
__device__ __forceinline__ void soa_dist4(const SoaStage& st, int j, f32x2 qx, f32x2 qy, f32x2 qz, float (&d)[4]) {
  const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(st.x + j);
  const ulonglong2 y = *reinterpret_cast<const ulonglong2*>(st.y + j);
  const ulonglong2 z = *reinterpret_cast<const ulonglong2*>(st.z + j);
  exact_dist2_x2(qx, qy, qz, x.x, y.x, z.x, d[0], d[1]);
  exact_dist2_x2(qx, qy, qz, x.y, y.y, z.y, d[2], d[3]);
}
__device__ __forceinline__ float4 soa_point(const SoaStage& st, int j) {
  return make_float4(st.x[j], st.y[j], st.z[j], __uint_as_float(st.i[j]));
}

// Visitor contract (per-lane state, warp-synchronous calls):
//   float metric(lo, hi)  warp-level pruning metric of a node (tile vs box)
//   bool  still(m)        node with metric m may still hold useful points
//   bool  need(lo, hi)    this lane needs the leaf
//   void  scan(stage)     this lane scans the 32 staged points (float4[32],
//                         or the SoaStage of a kSoa visitor)
//   void  visited(leaf)   warp-uniform notification after a leaf was scanned
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
      if (vis.skip(id)) continue;
      const float4 lo = ix.lo[0][id], hi = ix.hi[0][id];
      const bool need = vis.need(lo, hi);
      if (!__any_sync(LCR_FULL, need)) continue;
      scan_staged(ix, id, need, vis, ws);
      vis.visited(id);
      vis.refresh();
    } else {
      const int cl = level - 1;
      const int c = id * 32 + lane;
      bool has = c < ix.count[cl];
      float m = LCR_INF, dord = LCR_INF;
      if (has) {
        const float4 lo = ix.lo[cl][c], hi = ix.hi[cl][c];
        // An empty box (only non-finite points below it: lo = +inf, hi = -inf)
        // holds nothing and is never pushed.
        has = lo.x <= hi.x;
        m = vis.metric(lo, hi);
        // Visit order: box distance to the tile centre, ties (boxes containing
        // the centre, common for elongated leaves on grazing surfaces) broken
        // by the distance to the box centre.
        const float ox = 0.5f * (lo.x + hi.x) - cx, oy = 0.5f * (lo.y + hi.y) - cy, oz = 0.5f * (lo.z + hi.z) - cz;
        dord = box_dist2(lo, hi, cx, cy, cz) + 0.25f * (ox * ox + oy * oy + oz * oz);
        // The ranking below needs a strict total order: no NaN keys.
        if (!(dord <= LCR_INF)) dord = LCR_INF;
      }
      const bool pass = has && vis.still(m);
      const unsigned mask = __ballot_sync(LCR_FULL, pass);
      // Position among the passing children: farther children sit deeper in the
      // stack so the nearest is popped first.  Only passing lanes are compared
      // (usually a few, so the shuffle chain stays short).
      int pos = 0;
      for (unsigned mm = mask; mm; mm &= mm - 1u) {
        const int j = __ffs(mm) - 1;
        const float dj = __shfl_sync(LCR_FULL, dord, j);
        if (dj > dord || (dj == dord && j > lane)) ++pos;
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
// Only the (distance, index) key is carried through the scan; a caller that
// needs the point reads it by index afterwards (one load instead of four
// selects per candidate).
struct NN1 {
  float qx, qy, qz;
  bool qv;
  unsigned long long best;
  WarpScratch* ws;
  float R;

  __device__ __forceinline__ void init(float x, float y, float z, bool v, float cap, WarpScratch& w) {
    qx = x; qy = y; qz = z; qv = v;
    best = make_key(cap, 0xffffffffu);
    ws = &w;
    subtile_setup(x, y, z, v, w);
    refresh();
  }
  // Starts from a known candidate (warp-collective): the result is still the
  // exact nearest -- the candidate is one of the points -- but the search
  // prunes with its distance from the first node on.
  __device__ __forceinline__ void seed(unsigned long long k) {
    if (k < best) best = k;
    refresh();
  }
  __device__ __forceinline__ float bound() const { return key_dist(best); }
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return subtile_metric(lo, hi, *ws);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) <= bound();
  }
  // Four independent minimum chains over the 32 staged points, merged at the
  // end: keys are unique (the index is part of them), so the minimum is the
  // same whatever the grouping, and the loop no longer waits on one serial
  // compare-and-select chain.  The distances are computed two at a time in
  // paired FP32 (bit-identical to exact_dist2) from the coordinate-major stage.
  static constexpr bool kSoa = true;
  __device__ __forceinline__ void scan(const SoaStage& st) {
    const f32x2 qx2 = f32x2_dup(qx), qy2 = f32x2_dup(qy), qz2 = f32x2_dup(qz);
    unsigned long long b0 = best, b1 = best, b2 = best, b3 = best;
#pragma unroll
    for (int j = 0; j < 32; j += 4) {
      const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(st.x + j);
      const ulonglong2 y = *reinterpret_cast<const ulonglong2*>(st.y + j);
      const ulonglong2 z = *reinterpret_cast<const ulonglong2*>(st.z + j);
      const uint4 id = *reinterpret_cast<const uint4*>(st.i + j);
      float e0, e1, e2, e3;
      exact_dist2_x2(qx2, qy2, qz2, x.x, y.x, z.x, e0, e1);
      exact_dist2_x2(qx2, qy2, qz2, x.y, y.y, z.y, e2, e3);
      const unsigned long long k0 = make_key(e0, id.x);
      const unsigned long long k1 = make_key(e1, id.y);
      const unsigned long long k2 = make_key(e2, id.z);
      const unsigned long long k3 = make_key(e3, id.w);
      b0 = k0 < b0 ? k0 : b0;
      b1 = k1 < b1 ? k1 : b1;
      b2 = k2 < b2 ? k2 : b2;
      b3 = k3 < b3 ? k3 : b3;
    }
    b0 = b1 < b0 ? b1 : b0;
    b2 = b3 < b2 ? b3 : b2;
    best = b2 < b0 ? b2 : b0;
  }
  // Warp-collective form (every lane calls it).  When more than 16 lanes need
  // the leaf, each of them scans all 32 points (scan).  Otherwise the needing
  // lanes are spread over the warp: each is served by g = 2, 4 or 8 lanes
  // (the most that fit), which scan 32/g points apiece, and a shuffle tree
  // hands the owner its group's minimum key.  The minimum does not depend on
  // how the points are grouped, so the result is the same.
  static constexpr bool kWarpScan = true;
  __device__ __forceinline__ void scan_warp(const SoaStage& st, bool need) {
    const unsigned mask = __ballot_sync(LCR_FULL, need);
    const int nq = __popc(mask);
    if (nq > 16) {
      if (need) scan(st);
      return;
    }
    const int lane = threadIdx.x & 31;
    const int lg = nq <= 4 ? 3 : (nq <= 8 ? 2 : 1);    // log2 of the lanes per needing lane
    const int r = __popc(mask & ((1u << lane) - 1u));  // rank among the needing lanes
    if (need) ws->qown[r] = static_cast<uint8_t>(lane);
    __syncwarp();
    const int qi = lane >> lg;
    const int owner = qi < nq ? static_cast<int>(ws->qown[qi]) : lane;
    const f32x2 x2 = f32x2_dup(__shfl_sync(LCR_FULL, qx, owner));
    const f32x2 y2 = f32x2_dup(__shfl_sync(LCR_FULL, qy, owner));
    const f32x2 z2 = f32x2_dup(__shfl_sync(LCR_FULL, qz, owner));
    const int per = 32 >> lg;  // 16, 8 or 4 points
    const int j0 = (lane & ((1 << lg) - 1)) * per;
    unsigned long long b = ~0ull;
#pragma unroll 4
    for (int j = j0; j < j0 + per; j += 4) {
      float d[4];
      soa_dist4(st, j, x2, y2, z2, d);
      const uint4 id = *reinterpret_cast<const uint4*>(st.i + j);
      const unsigned long long k0 = make_key(d[0], id.x), k1 = make_key(d[1], id.y);
      const unsigned long long k2 = make_key(d[2], id.z), k3 = make_key(d[3], id.w);
      const unsigned long long m01 = k1 < k0 ? k1 : k0, m23 = k3 < k2 ? k3 : k2;
      const unsigned long long m = m23 < m01 ? m23 : m01;
      b = m < b ? m : b;
    }
    for (int o = 1; o < (1 << lg); o <<= 1) {
      const unsigned long long t = __shfl_xor_sync(LCR_FULL, b, o);
      b = t < b ? t : b;
    }
    const unsigned long long gb = __shfl_sync(LCR_FULL, b, (r << lg) & 31);
    if (need && gb < best) best = gb;
    __syncwarp();  // qown is rewritten at the next leaf
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() { R = subtile_radius(bound(), qv, *ws); }
  __device__ __forceinline__ bool found() const { return key_idx(best) != 0xffffffffu; }
};

// -------------------------------------------------- one query per warp
// Cooperative 1-NN of a single query: every lane tests one child box or one
// leaf point and the warp reduces the (distance, index) keys, so pruning is
// per query.  Same result as NN1 for that query: accepted iff distance <= cap,
// lowest index among ties.
struct WarpNN {
  float qx, qy, qz;
  unsigned long long best;
  float4 bp;
  float R;
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const { return box_dist2(lo, hi, qx, qy, qz); }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return box_dist2(lo, hi, qx, qy, qz) <= key_dist(best);
  }
  __device__ __forceinline__ void scan(const float4* st) {
    const int lane = threadIdx.x & 31;
    const float4 p = st[lane];
    const float d = exact_dist2(qx, qy, qz, p.x, p.y, p.z);
    // 32-bit minimum first (NaN sentinels lose: fminf ignores them); the index
    // only decides among exact distance ties.
    float dm = d;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dm = fminf(dm, __shfl_xor_sync(LCR_FULL, dm, o));
    if (!(dm <= key_dist(best))) return;
    const unsigned tie = __ballot_sync(LCR_FULL, d == dm);
    int src = __ffs(tie) - 1;
    uint32_t idx = __float_as_uint(__shfl_sync(LCR_FULL, p.w, src));
    for (unsigned t = tie & (tie - 1u); t; t &= t - 1u) {  // rare: equal distances
      const int j = __ffs(t) - 1;
      const uint32_t ij = __float_as_uint(__shfl_sync(LCR_FULL, p.w, j));
      if (ij < idx) {
        idx = ij;
        src = j;
      }
    }
    const unsigned long long k = make_key(dm, idx);
    if (k < best) {
      best = k;
      bp = st[src];
    }
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() { R = key_dist(best); }
};

__device__ __forceinline__ void warp_query_nn(const IndexView& ix, float qx, float qy, float qz, float cap,
                                              WarpScratch& ws, unsigned long long& best, float4& bp,
                                              unsigned long long seed = ~0ull, float4 seed_p = float4()) {
  WarpNN v;
  v.qx = qx; v.qy = qy; v.qz = qz;
  v.best = make_key(cap, 0xffffffffu);
  v.bp = make_float4(0.f, 0.f, 0.f, 0.f);
  if (seed < v.best) {  // a known candidate (warp-uniform): exact result, earlier pruning
    v.best = seed;
    v.bp = seed_p;
  }
  v.R = key_dist(v.best);
  tile_traverse(ix, v, qx, qy, qz, ws);
  best = v.best;
  bp = v.bp;
}

// Exact capped 1-NN for the warp's tile.  A tile much wider than the search
// radius (its 32 queries straddle a jump of the Hilbert order between distant
// surfaces) would admit most of the tree between its clusters, so it is split
// into its four 8-lane sub-tiles, each searched as a tile with the other lanes
// idle; a sub-tile that is still wide runs its queries one at a time through
// warp_query_nn.  Every path gives the same result per query.
__device__ __forceinline__ void tile_nn1(const IndexView& ix, float qx, float qy, float qz, bool qv, float cap,
                                         const float4& tlo, const float4& thi, WarpScratch& ws, NN1& v) {
  const float dx = thi.x - tlo.x, dy = thi.y - tlo.y, dz = thi.z - tlo.z;
  const float wide2 = 16.f * cap;
  if (!(dx * dx + dy * dy + dz * dz > wide2)) {
    v.init(qx, qy, qz, qv, cap, ws);
    tile_traverse(ix, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), ws);
    return;
  }
  const int lane = threadIdx.x & 31, grp = lane >> 3;
  unsigned long long best = make_key(cap, 0xffffffffu);
  for (int g = 0; g < 4; ++g) {
    const bool mine = qv && grp == g;
    float4 slo, shi;
    if (!tile_box(qx, qy, qz, mine, slo, shi)) continue;
    const float sx = shi.x - slo.x, sy = shi.y - slo.y, sz = shi.z - slo.z;
    if (!(sx * sx + sy * sy + sz * sz > wide2)) {
      NN1 s;
      s.init(qx, qy, qz, mine, cap, ws);
      tile_traverse(ix, s, 0.5f * (slo.x + shi.x), 0.5f * (slo.y + shi.y), 0.5f * (slo.z + shi.z), ws);
      if (mine) best = s.best;
    } else {
      const unsigned valid = __ballot_sync(LCR_FULL, mine);
      for (unsigned t = valid; t; t &= t - 1u) {
        const int l = __ffs(t) - 1;
        const float x = __shfl_sync(LCR_FULL, qx, l), y = __shfl_sync(LCR_FULL, qy, l), z = __shfl_sync(LCR_FULL, qz, l);
        unsigned long long b;
        float4 p;
        warp_query_nn(ix, x, y, z, cap, ws, b, p);
        if (lane == l) best = b;
      }
    }
  }
  v.qx = qx; v.qy = qy; v.qz = qz; v.qv = qv;
  v.best = best;
}

// ---------------------------------------------------------------- k-NN
// Exact k nearest neighbours per lane in two passes, without per-candidate
// sorted insertion (whose divergent shifting dominated):
//  pass 1: traverse; every lane bins candidate squared distances into a
//          log-spaced histogram (4 bins per octave) and keeps the bin b* that
//          holds its k-th smallest so far -- the bin's upper edge tau is a
//          running upper bound on the k-th distance that drives the pruning.
//          The warp records the leaves it scanned.
//  pass 2: rescan those leaves; each lane appends every candidate with
//          d <= tau (the count is known exactly from pass 1) and sorts the
//          buffer once.  A lane whose count would not fit keeps a sorted list
//          instead (rare: many points in the boundary bin, e.g. duplicates).
// The result is the exact first k keys in (distance, index) order, in
// list[j*32 + lane], j < k.
constexpr int kLeafList = 192;
constexpr int kSeedLeaves = 2;  // pass 1 first scans the query leaf and this many either side
constexpr int kBins = 64;  // 16 octaves of d^2, 8 of distance

__host__ __device__ constexpr int knn_buffer(int K) { return K + 32; }

struct KnnWarp {
  WarpScratch ws;
  uint32_t leaves[kLeafList];
};

// Bytes of shared memory one warp needs for k neighbours.
__host__ __device__ inline size_t knn_warp_bytes(int K) {
  const size_t buf = static_cast<size_t>(knn_buffer(K)) * 32 * 8;
  const size_t hist = static_cast<size_t>(kBins) * 32 * 4;
  return sizeof(KnnWarp) + (buf > hist ? buf : hist);
}

struct KHist {
  float qx, qy, qz;
  bool qv;
  int K, lane, e0, bs, cl, nleaves;
  float cap;
  uint32_t* hist;
  uint32_t* leaves;
  WarpScratch* ws;
  float R;
  float top_max;  // largest candidate binned into the last (open) bin
  // A lane whose k-th key falls in the open last bin has a bound that no longer
  // prunes (it is the farthest candidate seen).  With can_escape set, such a
  // lane leaves the tile (esc) once the seed leaves are scanned (seeded):
  // the caller searches it again on its own with a range from top_max, and the
  // tile keeps its compact radius.  Deciding only after the seeds keeps a lane
  // from leaving while it has met just its own leaf and one far neighbour.
  bool can_escape, esc, seeded;
  __device__ __forceinline__ bool should_escape() const { return can_escape && seeded && cl >= K && bs == kBins; }
  __device__ __forceinline__ void escape() {
    esc = true;
    qv = false;
  }

  __device__ __forceinline__ int bin(float d) const {
    const int b = static_cast<int>(__float_as_uint(d) >> 21) - e0;
    return min(max(b, 0), kBins - 1);
  }
  // Largest float of bin b; the last bin is open above, so its edge is the
  // largest candidate it received (a valid bound once the k-th lies in it).
  __device__ __forceinline__ float edge(int b) const {
    const int top = b + e0 + 1;
    if (b >= kBins - 1) return top_max;
    if (top >= 1020) return LCR_INF;
    return __uint_as_float((static_cast<uint32_t>(top) << 21) - 1u);
  }
  __device__ __forceinline__ float bound() const { return cl >= K ? fminf(edge(bs - 1), cap) : cap; }
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return subtile_metric(lo, hi, *ws);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) <= bound();
  }
  // Every staged point updates the lane's histogram without a branch (adding
  // 0 or 1 to its bin): a per-candidate branch ran for nearly every point,
  // since some lane of the warp usually takes it.  The bound is the one at
  // the start of the leaf and the top bins are dropped once after it.  The bin
  // that holds the k-th key, and every count below it, come out the same as
  // with per-candidate drops: a candidate above a bound that would have shrunk
  // within the leaf lands in a bin that is dropped.  When that bin is the open
  // last one, its count and edge (its largest candidate) can come out larger;
  // its range still holds the keys pass 2 selects from, so the k-set is
  // unchanged (tests/test_kset_pass1_model.py models both forms).
  static constexpr bool kSoa = true;
  __device__ __forceinline__ void scan(const SoaStage& st) {
    const float tau = bound();
    const f32x2 qx2 = f32x2_dup(qx), qy2 = f32x2_dup(qy), qz2 = f32x2_dup(qz);
    int add = 0;
    float tm = top_max;
    for (int j0 = 0; j0 < 32; j0 += 4) {
      float dd[4];
      soa_dist4(st, j0, qx2, qy2, qz2, dd);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float d = dd[u];
        const bool c = d <= tau;
        const int b = bin(d);
        hist[b * 32 + lane] += static_cast<uint32_t>(c);
        tm = (c && b == kBins - 1) ? fmaxf(tm, d) : tm;
        add += c;
      }
    }
    top_max = tm;
    if (add) {
      cl += add;
      if (cl >= K) {
        while (bs > 1) {
          const int top = static_cast<int>(hist[(bs - 1) * 32 + lane]);
          if (cl - top < K) break;
          cl -= top;
          --bs;
        }
        if (should_escape()) escape();
      }
    }
  }
  // Warp-collective form (every lane calls it).  When exactly one lane needs
  // the leaf (an escaped query searched alone, or a sparse corner of a tile),
  // the warp scans it for that lane, one point per lane: the same distances,
  // the same bound and the same 0-or-1 additions as scan(), so the same
  // histogram state, in one step instead of 32.
  static constexpr bool kWarpScan = true;
  __device__ __forceinline__ void scan_warp(const SoaStage& st, bool need) {
    const unsigned mask = __ballot_sync(LCR_FULL, need);
    if (__popc(mask) != 1) {
      if (need) scan(st);
      return;
    }
    const int owner = __ffs(mask) - 1;
    const float tau = __shfl_sync(LCR_FULL, bound(), owner);
    const int eo = __shfl_sync(LCR_FULL, e0, owner);
    const float x = __shfl_sync(LCR_FULL, qx, owner), y = __shfl_sync(LCR_FULL, qy, owner),
                z = __shfl_sync(LCR_FULL, qz, owner);
    const float d = exact_dist2(x, y, z, st.x[lane], st.y[lane], st.z[lane]);
    const bool c = d <= tau;
    const int b = min(max(static_cast<int>(__float_as_uint(d) >> 21) - eo, 0), kBins - 1);
    if (c) atomicAdd(&hist[b * 32 + owner], 1u);
    const int cnt = __popc(__ballot_sync(LCR_FULL, c));
    // largest candidate in the last bin: non-negative floats order as their bits
    const float tm = __uint_as_float(
        __reduce_max_sync(LCR_FULL, (c && b == kBins - 1) ? __float_as_uint(d) : 0u));
    __syncwarp();  // the additions before the owner reads its column
    if (lane == owner && cnt > 0) {
      top_max = fmaxf(top_max, tm);
      cl += cnt;
      if (cl >= K) {
        while (bs > 1) {
          const int top = static_cast<int>(hist[(bs - 1) * 32 + lane]);
          if (cl - top < K) break;
          cl -= top;
          --bs;
        }
        if (should_escape()) escape();
      }
    }
    __syncwarp();
  }
  // Leaves [seed_lo, seed_hi] were scanned before the traversal.
  int seed_lo, seed_hi;
  __device__ __forceinline__ bool skip(int id) const { return id >= seed_lo && id <= seed_hi; }
  __device__ __forceinline__ void visited(int id) {
    if (nleaves < kLeafList && lane == 0) leaves[nleaves] = static_cast<uint32_t>(id);
    ++nleaves;
  }
  // Scans one leaf outside the traversal (warp-uniform call).
  __device__ __forceinline__ void scan_leaf(const IndexView& ix, int id, WarpScratch& ws) {
    const float4 lo = ix.lo[0][id], hi = ix.hi[0][id];
    const bool nd = need(lo, hi);
    if (!__any_sync(LCR_FULL, nd)) return;
    scan_staged(ix, id, nd, *this, ws);
    visited(id);
    refresh();
  }
  __device__ __forceinline__ void refresh() { R = subtile_radius(bound(), qv, *ws); }
};

// Pass-2 collector over a fixed per-lane bound tau (re-traversal form, used
// when pass 1 scanned more leaves than the leaf list holds).
struct KCollect {
  float qx, qy, qz;
  bool qv, insert;
  int K, lane, cnt;
  float tau;
  unsigned long long* buf;
  WarpScratch* ws;
  float R;

  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return subtile_metric(lo, hi, *ws);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) <= tau;
  }
  static constexpr bool kSoa = true;
  __device__ __forceinline__ void scan(const SoaStage& st) {
    const f32x2 qx2 = f32x2_dup(qx), qy2 = f32x2_dup(qy), qz2 = f32x2_dup(qz);
    for (int j0 = 0; j0 < 32; j0 += 4) {
      float dd[4];
      soa_dist4(st, j0, qx2, qy2, qz2, dd);
      for (int u = 0; u < 4; ++u) {
        const float d = dd[u];
        if (!(d <= tau)) continue;
        const unsigned long long k = make_key(d, st.i[j0 + u]);
        if (!insert) {
          if (cnt < knn_buffer(K)) buf[cnt * 32 + lane] = k;  // fits by pass 1's count; bounded all the same
          ++cnt;
        } else if (k < buf[(K - 1) * 32 + lane]) {
          int pos = K - 1;
          while (pos > 0) {
            const unsigned long long prev = buf[(pos - 1) * 32 + lane];
            if (prev <= k) break;
            buf[pos * 32 + lane] = prev;
            --pos;
          }
          buf[pos * 32 + lane] = k;
        }
      }
    }
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() {}
};

// Pass 1 for the warp's tile (traversal + histogram, see KHist).  When the
// queries are the points of leaf `self_leaf` of ix itself, that leaf and its
// two neighbours on each side along the Hilbert order are scanned first: they
// settle the per-lane bounds before the traversal starts (16x fewer leaf visits
// on depth-camera clouds than traversal order alone).  self_leaf < 0: no
// seeding.  Afterwards kw.leaves holds the scanned leaves (h.nleaves of them).
__device__ __forceinline__ void knn_pass1(const IndexView& ix, float qx, float qy, float qz, bool qv, int K, float cap,
                                          const float4& tlo, const float4& thi, KnnWarp& kw, unsigned char* region,
                                          int self_leaf, KHist& h, float top_hint = 0.f, bool can_escape = false) {
  const int lane = threadIdx.x & 31;
  // Each lane's bins span 16 octaves of d^2 below min(16 x the tile diagonal,
  // 64 x the distance to the nearer of its two neighbours along the Hilbert
  // order)^2: the second term keeps the range local in a tile whose queries
  // straddle distant surfaces (there the tile diagonal would push every
  // neighbour into the lowest, clamped bin).
  const float dx = thi.x - tlo.x, dy = thi.y - tlo.y, dz = thi.z - tlo.z;
  float top2 = 256.f * (dx * dx + dy * dy + dz * dz);
  {
    const float ux = __shfl_up_sync(LCR_FULL, qx, 1), uy = __shfl_up_sync(LCR_FULL, qy, 1),
                uz = __shfl_up_sync(LCR_FULL, qz, 1);
    const float wx = __shfl_down_sync(LCR_FULL, qx, 1), wy = __shfl_down_sync(LCR_FULL, qy, 1),
                wz = __shfl_down_sync(LCR_FULL, qz, 1);
    const bool uv = __shfl_up_sync(LCR_FULL, qv, 1) && lane > 0;
    const bool wv = __shfl_down_sync(LCR_FULL, qv, 1) && lane < 31;
    float sp = LCR_INF;
    if (qv && uv) sp = exact_dist2(qx, qy, qz, ux, uy, uz);
    if (qv && wv) sp = fminf(sp, exact_dist2(qx, qy, qz, wx, wy, wz));
    if (sp > 0.f && sp < LCR_INF) top2 = fminf(top2, 4096.f * sp);
  }
  if (top_hint > 0.f) top2 = top_hint;  // the caller knows the lane's scale
  top2 = fmaxf(top2, 1e-30f);
  h.qx = qx; h.qy = qy; h.qz = qz; h.qv = qv;
  h.K = K; h.lane = lane;
  h.e0 = static_cast<int>(__float_as_uint(top2) >> 21) - (kBins - 1);
  h.bs = kBins; h.cl = 0; h.nleaves = 0; h.top_max = 0.f;
  h.can_escape = can_escape;
  h.esc = false;
  h.seeded = self_leaf < 0;
  h.cap = cap;
  h.hist = reinterpret_cast<uint32_t*>(region);
  h.leaves = kw.leaves;
  h.ws = &kw.ws;
  for (int b = 0; b < kBins; ++b) h.hist[b * 32 + lane] = 0u;
  h.seed_lo = 1;
  h.seed_hi = 0;
  subtile_setup(qx, qy, qz, qv, kw.ws);
  h.refresh();
  if (self_leaf >= 0) {
    // the traversal skips exactly the leaves scanned here: one constant for both
    h.seed_lo = max(0, self_leaf - kSeedLeaves);
    h.seed_hi = min(ix.nleaf - 1, self_leaf + kSeedLeaves);
    h.scan_leaf(ix, self_leaf, kw.ws);
    for (int d = 1; d <= kSeedLeaves; ++d) {
      if (self_leaf - d >= 0) h.scan_leaf(ix, self_leaf - d, kw.ws);
      if (self_leaf + d < ix.nleaf) h.scan_leaf(ix, self_leaf + d, kw.ws);
    }
    h.seeded = true;
    if (h.should_escape()) h.escape();
    h.refresh();
  }
  tile_traverse(ix, h, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), kw.ws);
  __syncwarp();
}

// Pass 2 over the leaves pass 1 scanned (or a re-traversal when they did not
// fit the leaf list).  vis.need() is re-evaluated per leaf with the final bound.
template <class V>
__device__ __forceinline__ void knn_pass2(const IndexView& ix, const KHist& h, V& vis, const float4& tlo,
                                          const float4& thi, KnnWarp& kw) {
  if (h.nleaves <= kLeafList) {
    for (int l = 0; l < h.nleaves; ++l) {
      const int id = static_cast<int>(kw.leaves[l]);
      const float4 lo = ix.lo[0][id], hi = ix.hi[0][id];
      const bool nd = vis.need(lo, hi);
      if (!__any_sync(LCR_FULL, nd)) continue;
      scan_staged(ix, id, nd, vis, kw.ws);
    }
  } else {
    tile_traverse(ix, vis, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), kw.ws);
  }
  __syncwarp();
}

// Runs both passes for the warp's tile.  Afterwards list = region as
// unsigned long long [.][32] holds each lane's sorted k nearest keys in its
// first K rows (missing entries: key (inf, 0xffffffff)).
__device__ __forceinline__ void tile_knn(const IndexView& ix, float qx, float qy, float qz, bool qv, int K, float cap,
                                         const float4& tlo, const float4& thi, KnnWarp& kw, unsigned char* region,
                                         int self_leaf = -1, float top_hint = 0.f) {
  const int lane = threadIdx.x & 31;
  KHist h;
  knn_pass1(ix, qx, qy, qz, qv, K, cap, tlo, thi, kw, region, self_leaf, h, top_hint);
  const float tau = h.bound();
  const int cnt = h.cl;
  KCollect c;
  c.qx = qx; c.qy = qy; c.qz = qz; c.qv = qv;
  c.K = K; c.lane = lane; c.cnt = 0; c.tau = tau;
  c.insert = cnt > knn_buffer(K);
  c.buf = reinterpret_cast<unsigned long long*>(region);
  c.ws = &kw.ws;
  c.R = subtile_radius(tau, qv, kw.ws);
  const unsigned long long none = make_key(LCR_INF, 0xffffffffu);
  if (c.insert)
    for (int j = 0; j < K; ++j) c.buf[j * 32 + lane] = none;
  __syncwarp();
  knn_pass2(ix, h, c, tlo, thi, kw);
  if (!c.insert) {
    unsigned long long* b = c.buf;
    const int n = c.cnt;
    for (int i = 1; i < n; ++i) {
      const unsigned long long k = b[i * 32 + lane];
      int j = i;
      while (j > 0) {
        const unsigned long long prev = b[(j - 1) * 32 + lane];
        if (prev <= k) break;
        b[j * 32 + lane] = prev;
        --j;
      }
      b[j * 32 + lane] = k;
    }
    for (int j = n; j < K; ++j) b[j * 32 + lane] = none;
  }
  __syncwarp();
}

// ------------------------------------------------ unordered k-NN reductions
// Statistics over the set of k nearest neighbours (a sum, a covariance) need
// the set, not its order.  After pass 1 every lane knows the bin holding its
// k-th key and the count of candidates in lower bins; those are all among the
// k nearest.  The boundary is kept as a key range [klo, khi] with the number m
// of keys still needed from it.  While some lane's range holds more than
// kBoundCap candidates (equal or nearly equal distances, a clamped bin), a
// refinement pass splits the range into 64 sub-ranges of the (distance, index)
// key and keeps the one holding the m-th key (radix selection: keys are unique,
// so this ends).  The collect pass then hands every key below klo to an
// accumulator and buffers the boundary keys, from which the m smallest are
// selected exactly.  No per-lane sorted list: about half the shared memory of
// tile_knn and no O(k^2) sort.
constexpr int kBoundCap = 32;  // boundary keys kept per lane: 8 KB per warp, as the histogram
constexpr int kRefineBits = 6;  // a refinement pass splits the boundary range into 64 sub-ranges
static_assert((1 << kRefineBits) <= kBins, "refinement sub-ranges must fit the histogram region");

__host__ __device__ inline size_t kset_warp_bytes() {
  const size_t buf = static_cast<size_t>(kBoundCap) * 32 * 8;
  const size_t hist = static_cast<size_t>(kBins) * 32 * 4;
  return sizeof(KnnWarp) + (buf > hist ? buf : hist);
}

// Pruning radius of a boundary key range: its largest distance.
__device__ __forceinline__ float range_tau(unsigned long long khi) { return key_dist(khi); }

// Refinement pass: per-lane histogram of the keys in [klo, khi] over 64
// sub-ranges of width 2^sh (lanes with active == false only follow along).
struct KRefine {
  float qx, qy, qz;
  bool qv, active;
  int lane, sh;
  unsigned long long klo, khi;
  float tau;
  uint32_t* hist;
  WarpScratch* ws;
  float R;
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return subtile_metric(lo, hi, *ws);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return active && box_dist2(lo, hi, qx, qy, qz) <= tau;
  }
  static constexpr bool kSoa = true;
  __device__ __forceinline__ void scan(const SoaStage& st) {
    const f32x2 qx2 = f32x2_dup(qx), qy2 = f32x2_dup(qy), qz2 = f32x2_dup(qz);
    for (int j0 = 0; j0 < 32; j0 += 4) {
      float dd[4];
      soa_dist4(st, j0, qx2, qy2, qz2, dd);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float d = dd[u];
        if (!(d <= tau)) continue;
        const unsigned long long k = make_key(d, st.i[j0 + u]);
        if (k < klo || k > khi) continue;
        hist[static_cast<int>((k - klo) >> sh) * 32 + lane] += 1u;
      }
    }
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() {}
};

// Collect pass: keys below klo go to the accumulator, keys in [klo, khi] to
// the boundary buffer.
template <class Acc>
struct KSet {
  float qx, qy, qz;
  bool qv;
  int lane, nb;
  unsigned long long klo, khi;
  float tau;
  unsigned long long* bbuf;
  Acc* acc;
  WarpScratch* ws;
  float R;

  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    return subtile_metric(lo, hi, *ws);
  }
  __device__ __forceinline__ bool still(float m) const { return m <= R; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && box_dist2(lo, hi, qx, qy, qz) <= tau;
  }
  static constexpr bool kSoa = true;
  __device__ __forceinline__ void scan(const SoaStage& st) {
    const f32x2 qx2 = f32x2_dup(qx), qy2 = f32x2_dup(qy), qz2 = f32x2_dup(qz);
    for (int j0 = 0; j0 < 32; j0 += 4) {
      float dd[4];
      soa_dist4(st, j0, qx2, qy2, qz2, dd);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
      const float d = dd[u];
      if (!(d <= tau)) continue;
      const unsigned long long k = make_key(d, st.i[j0 + u]);
      if (k < klo) {
        acc->add(soa_point(st, j0 + u), d);
      } else if (k <= khi) {
        if (nb < kBoundCap) bbuf[nb * 32 + lane] = k;
        ++nb;
      }
      }
    }
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() {}
};

// Feeds the k nearest points of each valid lane (exact set under the
// (distance, index) order; all points if the cloud holds fewer than k) to acc.
// top_hint > 0 sets the top of the lanes' histogram range (squared distance).
// acc.begin(tau, k) with the largest squared distance that can be fed, then
// acc.add(point, d) for points met in the collect pass and acc.add_key(key)
// for the selected boundary keys.  Queries are the points of leaf self_leaf of ix.
// With escape non-null, a lane whose k-th key lies above its histogram range
// leaves the tile (see KHist): *escape is set, its accumulator gets nothing,
// and *escape_top holds the largest squared distance it met -- at least its
// k-th -- for the caller's second search of that query.
template <class Acc>
__device__ __forceinline__ void tile_kset(const IndexView& ix, float qx, float qy, float qz, bool qv, int K,
                                          const float4& tlo, const float4& thi, KnnWarp& kw, unsigned char* region,
                                          int self_leaf, Acc& acc, float top_hint = 0.f, bool* escape = nullptr,
                                          float* escape_top = nullptr) {
  const int lane = threadIdx.x & 31;
  KHist h;
  knn_pass1(ix, qx, qy, qz, qv, K, LCR_INF, tlo, thi, kw, region, self_leaf, h, top_hint, escape != nullptr);
  if (escape) {
    *escape = h.esc;
    if (escape_top) *escape_top = h.top_max;
    qv = qv && !h.esc;
  }
  // boundary range: the bin holding the k-th key (everything if fewer than k)
  unsigned long long klo = make_key(LCR_INF, 0xffffffffu), khi = klo;  // fewer than k: every key is below klo
  int m = 0, cnt = 0;
  if (qv && h.cl >= K) {
    const int b = h.bs - 1;
    cnt = static_cast<int>(h.hist[b * 32 + lane]);
    m = K - (h.cl - cnt);
    klo = b == 0 ? 0ull : make_key(h.edge(b - 1), 0xffffffffu) + 1ull;
    khi = make_key(h.edge(b), 0xffffffffu);
  }
  __syncwarp();
  uint32_t* hist = reinterpret_cast<uint32_t*>(region);
  while (__any_sync(LCR_FULL, cnt > kBoundCap)) {
    KRefine r;
    r.qx = qx; r.qy = qy; r.qz = qz; r.qv = qv;
    r.active = cnt > kBoundCap;
    r.lane = lane;
    const unsigned long long span = khi - klo;  // >= cnt - 1 >= kBoundCap: keys are unique
    // (k - klo) >> sh <= span >> sh < 2^kRefineBits
    r.sh = r.active ? max(0, 64 - __clzll(static_cast<long long>(span)) - kRefineBits) : 0;
    r.klo = klo; r.khi = khi;
    r.tau = r.active ? range_tau(khi) : -1.f;
    r.hist = hist;
    r.ws = &kw.ws;
    r.R = subtile_radius(r.tau, r.active, kw.ws);
    for (int b = 0; b < (1 << kRefineBits); ++b) hist[b * 32 + lane] = 0u;
    __syncwarp();
    knn_pass2(ix, h, r, tlo, thi, kw);
    if (r.active) {
      int c = 0;
      for (int j = 0; j < (1 << kRefineBits); ++j) {
        const int hj = static_cast<int>(hist[j * 32 + lane]);
        if (c + hj >= m) {
          const unsigned long long lo = klo + (static_cast<unsigned long long>(j) << r.sh);
          const unsigned long long top = lo + ((1ull << r.sh) - 1ull);
          klo = lo;
          if (top < khi && top >= lo) khi = top;
          m -= c;
          cnt = hj;
          break;
        }
        c += hj;
      }
    }
    __syncwarp();
  }
  KSet<Acc> s;
  s.qx = qx; s.qy = qy; s.qz = qz; s.qv = qv;
  s.lane = lane; s.nb = 0;
  s.klo = klo; s.khi = khi;
  s.tau = qv ? range_tau(khi) : -1.f;
  s.bbuf = reinterpret_cast<unsigned long long*>(region);
  s.acc = &acc;
  s.ws = &kw.ws;
  s.R = subtile_radius(s.tau, qv, kw.ws);
  acc.begin(s.tau, K);
  knn_pass2(ix, h, s, tlo, thi, kw);
  if (qv && m > 0) {
    // partial selection sort: the m smallest of the nb (<= kBoundCap) boundary keys
    unsigned long long* b = s.bbuf;
    const int nb = min(s.nb, kBoundCap);
    for (int i = 0; i < m && i < nb; ++i) {
      int arg = i;
      unsigned long long best = b[i * 32 + lane];
      for (int j = i + 1; j < nb; ++j) {
        const unsigned long long k = b[j * 32 + lane];
        if (k < best) {
          best = k;
          arg = j;
        }
      }
      b[arg * 32 + lane] = b[i * 32 + lane];
      b[i * 32 + lane] = best;
      acc.add_key(best);
    }
  }
  __syncwarp();
}
