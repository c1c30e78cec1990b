// StatisticalOutlierRemoval, NormalEstimation and the accumulate_clouds crop
// predicate, each fused into the epilogue of the warp-tile neighbour search.
#include <algorithm>
#include <cmath>

#include "search.cuh"

namespace {

// Lanes whose k-th neighbour lies above their histogram range (isolated
// points: a fragment far from the rest) leave their tile and are queued with
// the largest squared distance they met; k_normals_escaped searches each of
// them alone with a range that holds its k-th (k_sor_dist_escaped for SOR).
// One such lane used to make its whole warp traverse the cloud, with a bound
// that did not prune.
struct EscapeQueue {
  uint32_t* slot;   // sorted slot of the query in the index
  float* top;       // largest squared distance met before leaving (>= its k-th)
  unsigned int* n;
};

__device__ __forceinline__ void escape_push(const EscapeQueue& q, uint32_t slot, float top) {
  const unsigned i = atomicAdd(q.n, 1u);
  q.slot[i] = slot;
  q.top[i] = top;
}

// ------------------------------------------------------------------ SOR
// outlier_removal.cpp:80-84.  kNN with k+1 results (the query itself first),
// mean of sqrt(d) over results 1..k summed in double in ascending order
// (float sqrt, as std::sqrt on a float), stored as float.
//
// Fast form: the k+1 nearest as an unordered set (tile_kset).  The ascending
// double sum equals the exact sum, in any order, whenever no partial sum can
// round: all terms are non-negative multiples of u = the smallest ulp among the
// nonzero float terms, so every partial sum is a multiple of u no larger than
// the total T, and T < 2^53 u makes all of them representable.  Then
// sum(results 1..k) = T - sqrt(d_min) exactly.  The terms are added exactly as
// 64-bit integers on a grid of 2^eg below the largest possible term (integer
// adds instead of FP64 ones); a term below that grid, or a lane that fails the
// test (a dynamic range above ~2^23 between neighbour distances), sends the
// tile to k_sor_dist_sorted.
struct SorAcc {
  long long sum;  // exact sum in units of 2^eg
  int eg;         // grid exponent
  float dmin;
  int emin;       // smallest biased exponent (>= 1) of a nonzero term
  int cnt;
  bool off_grid;
  __device__ __forceinline__ void init(unsigned long long* list) {
    out = list;
    sum = 0;
    eg = 0;
    dmin = LCR_INF;
    emin = 255;
    cnt = 0;
    off_grid = false;
  }
  // tau bounds every d to be added: terms are <= sqrt(tau) < 2^(E+24) with
  // E = exponent of sqrt(tau) - 150; a term shifted onto the grid stays below
  // 2^56 and k of them below 2^63 for k < 128 (the shift shrinks beyond).
  __device__ __forceinline__ void begin(float tau, int K) {
    kcap = K;
    const int e = static_cast<int>(__float_as_uint(__fsqrt_rn(tau)) >> 23);
    int lg = 0;
    while ((1 << lg) < K) ++lg;
    eg = max(e, 1) - 150 - (38 - lg);
  }
  __device__ __forceinline__ long long units(float v) {
    const uint32_t bits = __float_as_uint(v);
    const int e = static_cast<int>(bits >> 23);
    const long long man = e ? static_cast<long long>((bits & 0x7fffffu) | 0x800000u) : static_cast<long long>(bits);
    const int sh = max(e, 1) - 150 - eg;
    if (sh < 0 || sh > 39) {
      off_grid = true;
      return 0;
    }
    return man << sh;
  }
  __device__ __forceinline__ void add_d(float d) {
    const float v = __fsqrt_rn(d);
    ++cnt;
    dmin = fminf(dmin, d);
    if (v > 0.f) {
      sum += units(v);
      emin = min(emin, max(1, static_cast<int>(__float_as_uint(v) >> 23)));
    }
  }
  // the neighbour list of the query (may be null): the keys as they come.  The
  // k-set hands over exactly K keys; the write is bounded all the same, so that
  // no error upstream can write past the list.
  unsigned long long* out;
  int kcap = 0;
  __device__ __forceinline__ void add(const float4& p, float d) {
    if (out && cnt < kcap) out[cnt] = make_key(d, __float_as_uint(p.w));
    add_d(d);
  }
  __device__ __forceinline__ void add_key(unsigned long long k) {
    if (out && cnt < kcap) out[cnt] = k;
    add_d(key_dist(k));
  }
  // true if the ascending double sum is the exact one; s = that sum of all
  // terms but the smallest
  __device__ __forceinline__ bool result(double& s) {
    if (off_grid) return false;
    // T < 2^53 u, u = 2^(emin - 150) = 2^(emin - 150 - eg) grid units
    const int lim = 53 + emin - 150 - eg;
    if (emin < 255 && lim < 63 && sum >= (1ll << lim)) return false;
    const float vmin = __fsqrt_rn(dmin);
    const long long t = sum - (vmin > 0.f ? units(vmin) : 0ll);
    if (off_grid) return false;
    s = __dmul_rn(__ll2double_rn(t), __longlong_as_double(static_cast<long long>(eg + 1023) << 52));
    return true;
  }
};

__device__ __forceinline__ void sor_store(const float4& q, double s, int mean_k, float* __restrict__ dist,
                                          uint8_t* __restrict__ valid, unsigned int* __restrict__ nvalid) {
  const uint32_t o = __float_as_uint(q.w);
  dist[o] = __double2float_rn(__ddiv_rn(s, static_cast<double>(mean_k)));
  valid[o] = 1;
  atomicAdd(nvalid, 1u);
}

// too_few is set when a query has fewer than k+1 neighbours (the cloud holds
// at most k finite points); the host reports it after the pass.
__global__ void k_sor_dist(IndexView ix, int mean_k, float* __restrict__ dist, uint8_t* __restrict__ valid,
                           unsigned int* __restrict__ nvalid, uint32_t* __restrict__ redo, unsigned int* nredo,
                           int* too_few, unsigned long long* __restrict__ lists, EscapeQueue eq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int K = mean_k + 1;
  unsigned char* wbase = smem + wib * kset_warp_bytes();
  const int tile = blockIdx.x * nw + wib;
  if (tile >= ix.nleaf) return;
  const float4 q = ix.pts[static_cast<size_t>(tile) * 32 + lane];
  const bool qv = finite3(q.x, q.y, q.z);
  float4 tlo, thi;
  if (!tile_box(q.x, q.y, q.z, qv, tlo, thi)) return;
  SorAcc acc;
  acc.init(lists && qv ? lists + static_cast<size_t>(__float_as_uint(q.w)) * K : nullptr);
  bool esc = false;
  float top = 0.f;
  tile_kset(ix, q.x, q.y, q.z, qv, K, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), wbase + sizeof(KnnWarp), tile,
            acc, 0.f, &esc, &top);
  const bool mine = qv && !esc;
  if (mine && acc.cnt < K) *too_few = 1;
  double s = 0.0;
  if (!__all_sync(LCR_FULL, !mine || acc.result(s))) {
    // the sorted form redoes the whole tile, escaped lanes included
    if (lane == 0) redo[atomicAdd(nredo, 1u)] = static_cast<uint32_t>(tile);
    return;
  }
  if (mine) sor_store(q, s, mean_k, dist, valid, nvalid);
  if (esc) escape_push(eq, static_cast<uint32_t>(tile) * 32u + lane, top);
}

// The escaped SOR queries, one warp each (warps stride over the queue): the
// sorted k-NN of the query alone (tile_knn, the ascending double sum of the
// sorted form), its histogram topped at four times the largest squared
// distance it met, seeded with its own leaf and two either side.
__global__ void k_sor_dist_escaped(IndexView ix, int mean_k, float* __restrict__ dist, uint8_t* __restrict__ valid,
                                   unsigned int* __restrict__ nvalid, unsigned long long* __restrict__ lists,
                                   EscapeQueue eq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int K = mean_k + 1;
  unsigned char* wbase = smem + wib * knn_warp_bytes(K);
  unsigned char* region = wbase + sizeof(KnnWarp);
  const unsigned long long* list = reinterpret_cast<const unsigned long long*>(region);
  const unsigned int count = *eq.n;
  for (unsigned int w = blockIdx.x * nw + wib; w < count; w += gridDim.x * nw) {
    const uint32_t slot = eq.slot[w];
    const float4 p = ix.pts[slot];
    const bool qv = lane == 0;
    const float qx = qv ? p.x : 0.f, qy = qv ? p.y : 0.f, qz = qv ? p.z : 0.f;
    float4 tlo, thi;
    tile_box(qx, qy, qz, qv, tlo, thi);
    tile_knn(ix, qx, qy, qz, qv, K, LCR_INF, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), region,
             static_cast<int>(slot >> 5), 4.f * fmaxf(eq.top[w], 1e-30f));
    if (qv) {
      double s = 0.0;
      for (int j = 1; j < K; ++j) s = __dadd_rn(s, static_cast<double>(__fsqrt_rn(key_dist(list[j * 32]))));
      sor_store(p, s, mean_k, dist, valid, nvalid);
      if (lists)
        for (int j = 0; j < K; ++j) lists[static_cast<size_t>(__float_as_uint(p.w)) * K + j] = list[j * 32];
    }
    __syncwarp();
  }
}

// Sorted form for the queued tiles: the ascending double sum over the sorted
// k+1 nearest, one warp per tile, warps striding over the queue.
__global__ void k_sor_dist_sorted(IndexView ix, int mean_k, float* __restrict__ dist, uint8_t* __restrict__ valid,
                                  unsigned int* __restrict__ nvalid, const uint32_t* __restrict__ redo,
                                  const unsigned int* nredo, unsigned long long* __restrict__ lists) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int K = mean_k + 1;
  unsigned char* wbase = smem + wib * knn_warp_bytes(K);
  unsigned char* region = wbase + sizeof(KnnWarp);
  const unsigned long long* list = reinterpret_cast<const unsigned long long*>(region);
  const unsigned int count = *nredo;
  for (unsigned int i = blockIdx.x * nw + wib; i < count; i += gridDim.x * nw) {
    const int tile = static_cast<int>(redo[i]);
    const float4 q = ix.pts[static_cast<size_t>(tile) * 32 + lane];
    const bool qv = finite3(q.x, q.y, q.z);
    float4 tlo, thi;
    if (!tile_box(q.x, q.y, q.z, qv, tlo, thi)) continue;
    tile_knn(ix, q.x, q.y, q.z, qv, K, LCR_INF, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), region, tile);
    if (qv) {
      double s = 0.0;
      for (int j = 1; j < K; ++j) s = __dadd_rn(s, static_cast<double>(__fsqrt_rn(key_dist(list[j * 32 + lane]))));
      sor_store(q, s, mean_k, dist, valid, nvalid);
      if (lists)
        for (int j = 0; j < K; ++j) lists[static_cast<size_t>(__float_as_uint(q.w)) * K + j] = list[j * 32 + lane];
    }
    __syncwarp();
  }
}

// Fixed blocked order, one warp per chunk of 256 consecutive terms: lane l
// adds terms 8l .. 8l+7 of the chunk in order from 0.0, then the lanes combine
// by the xor butterfly 16, 8, 4, 2, 1 and lane 0's value is the chunk's sum
// (level 0 sums d and float(d*d)); repeated until one value remains.
__device__ __forceinline__ double butterfly_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(LCR_FULL, v, o));
  return v;
}

__global__ void k_bsum_level0(const float* __restrict__ d, int n, double* __restrict__ oa, double* __restrict__ ob) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int b = c * 256;
  if (b >= n) return;
  double sa = 0.0, sb = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int i = b + lane * 8 + j;
    if (i < n) {
      const float v = d[i];
      sa = __dadd_rn(sa, static_cast<double>(v));
      sb = __dadd_rn(sb, static_cast<double>(__fmul_rn(v, v)));
    }
  }
  sa = butterfly_sum(sa);
  sb = butterfly_sum(sb);
  if (lane == 0) {
    oa[c] = sa;
    ob[c] = sb;
  }
}

__global__ void k_bsum_level(const double* __restrict__ a, const double* __restrict__ b, int n,
                             double* __restrict__ oa, double* __restrict__ ob) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int s0 = c * 256;
  if (s0 >= n) return;
  double sa = 0.0, sb = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int i = s0 + lane * 8 + j;
    if (i < n) {
      sa = __dadd_rn(sa, a[i]);
      sb = __dadd_rn(sb, b[i]);
    }
  }
  sa = butterfly_sum(sa);
  sb = butterfly_sum(sb);
  if (lane == 0) {
    oa[c] = sa;
    ob[c] = sb;
  }
}

// mean = sum/nv; variance = (sq - sum*sum/nv)/(nv-1); threshold = mean + mul*stddev.
__global__ void k_sor_threshold(const double* __restrict__ sum, const double* __restrict__ sq,
                                const unsigned int* __restrict__ nvalid, double mul, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  const double nv = static_cast<double>(*nvalid);
  const double mean = __ddiv_rn(*sum, nv);
  const double var = __ddiv_rn(__dsub_rn(*sq, __ddiv_rn(__dmul_rn(*sum, *sum), nv)), __dsub_rn(nv, 1.0));
  const double sd = __dsqrt_rn(var);
  out[0] = mean;
  out[1] = sd;
  out[2] = __dadd_rn(mean, __dmul_rn(mul, sd));
}

__global__ void k_sor_flags(const float* __restrict__ dist, int n, const double* __restrict__ stats,
                            uint8_t* __restrict__ keep, uint8_t* __restrict__ drop) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool out = static_cast<double>(dist[i]) > stats[2];
  keep[i] = out ? 0 : 1;
  drop[i] = out ? 1 : 0;
}

// -------------------------------------------------------------- normals
// Smallest eigenpair of a symmetric 3x3 (FP64): FP32 trigonometric estimate of
// the smallest root of the characteristic cubic, Newton refinement in FP64, and
// the eigenvector as the best-conditioned cross product of two rows of A - l*I.
// Everything stays in registers: scalars and selects, no arrays indexed at run
// time (those went to the stack, ~200 bytes of local-memory traffic per point).
struct Eig3 {
  double lam, n0, n1, n2;
};

__device__ __forceinline__ Eig3 smallest_eig(double c00, double c01, double c02, double c11, double c12, double c22) {
  Eig3 r;
  const double s = fmax(fmax(fmax(fabs(c00), fabs(c01)), fmax(fabs(c02), fabs(c11))), fmax(fabs(c12), fabs(c22)));
  if (!(s > 0.0)) {
    // all neighbours coincide: no plane (PCL's eigen33 divides 0 by 0 here)
    r.lam = 0.0;
    r.n0 = r.n1 = r.n2 = __longlong_as_double(0x7ff8000000000000ll);
    return r;
  }
  const double a00 = c00 / s, a01 = c01 / s, a02 = c02 / s, a11 = c11 / s, a12 = c12 / s, a22 = c22 / s;
  const double c2 = a00 + a11 + a22;
  const double c1 = a00 * a11 + a00 * a22 + a11 * a22 - a01 * a01 - a02 * a02 - a12 * a12;
  const double c0 = a00 * (a11 * a22 - a12 * a12) - a01 * (a01 * a22 - a12 * a02) + a02 * (a01 * a12 - a11 * a02);
  // FP32 estimate (trigonometric solution of the depressed cubic)
  float l0;
  {
    const float q = static_cast<float>(c2) / 3.f;
    const float b00 = static_cast<float>(a00) - q, b11 = static_cast<float>(a11) - q, b22 = static_cast<float>(a22) - q;
    const float f01 = static_cast<float>(a01), f02 = static_cast<float>(a02), f12 = static_cast<float>(a12);
    const float p1 = f01 * f01 + f02 * f02 + f12 * f12;
    const float p2 = b00 * b00 + b11 * b11 + b22 * b22 + 2.f * p1;
    const float p = sqrtf(p2 / 6.f);
    if (p > 0.f) {
      const float ip = 1.f / p;
      const float B00 = b00 * ip, B11 = b11 * ip, B22 = b22 * ip, B01 = f01 * ip, B02 = f02 * ip, B12 = f12 * ip;
      float rr = 0.5f * (B00 * (B11 * B22 - B12 * B12) - B01 * (B01 * B22 - B12 * B02) + B02 * (B01 * B12 - B11 * B02));
      rr = fminf(1.f, fmaxf(-1.f, rr));
      const float phi = acosf(rr) / 3.f;
      l0 = q + 2.f * p * cosf(phi + 2.0943951f);
    } else {
      l0 = q;
    }
  }
  double l = l0;
  for (int it = 0; it < 4; ++it) {
    const double f = ((-l + c2) * l - c1) * l + c0;       // det(A - l I)
    const double fp = (-3.0 * l + 2.0 * c2) * l - c1;     // derivative
    if (!(fabs(fp) > 0.0)) break;
    const double step = f / fp;
    l -= step;
    if (fabs(step) <= 1e-17 * fmax(1.0, fabs(l))) break;
  }
  // rows of A - l I
  const double r00 = a00 - l, r01 = a01, r02 = a02;
  const double r10 = a01, r11 = a11 - l, r12 = a12;
  const double r20 = a02, r21 = a12, r22 = a22 - l;
  // cross products of row pairs (0,1), (0,2), (1,2); the largest is the best conditioned
  const double x00 = r01 * r12 - r02 * r11, x01 = r02 * r10 - r00 * r12, x02 = r00 * r11 - r01 * r10;
  const double x10 = r01 * r22 - r02 * r21, x11 = r02 * r20 - r00 * r22, x12 = r00 * r21 - r01 * r20;
  const double x20 = r11 * r22 - r12 * r21, x21 = r12 * r20 - r10 * r22, x22 = r10 * r21 - r11 * r20;
  const double m0 = x00 * x00 + x01 * x01 + x02 * x02, m1 = x10 * x10 + x11 * x11 + x12 * x12,
               m2 = x20 * x20 + x21 * x21 + x22 * x22;
  double bn = m0, b0 = x00, b1 = x01, b2 = x02;
  if (m1 > bn) { bn = m1; b0 = x10; b1 = x11; b2 = x12; }
  if (m2 > bn) { bn = m2; b0 = x20; b1 = x21; b2 = x22; }
  if (bn > 1e-28) {
    const double inv = 1.0 / sqrt(bn);
    r.n0 = b0 * inv; r.n1 = b1 * inv; r.n2 = b2 * inv;
  } else {
    // A - l I has rank <= 1: any unit vector orthogonal to its largest row.
    const double q0 = r00 * r00 + r01 * r01 + r02 * r02, q1 = r10 * r10 + r11 * r11 + r12 * r12,
                 q2 = r20 * r20 + r21 * r21 + r22 * r22;
    double qn = q0, g0 = r00, g1 = r01, g2 = r02;
    if (q1 > qn) { qn = q1; g0 = r10; g1 = r11; g2 = r12; }
    if (q2 > qn) { qn = q2; g0 = r20; g1 = r21; g2 = r22; }
    // the axis of the row's smallest component
    const bool ax0 = fabs(g0) <= fabs(g1) && fabs(g0) <= fabs(g2);
    const bool ax1 = !ax0 && fabs(g1) <= fabs(g2);
    const double e0 = ax0 ? 1.0 : 0.0, e1 = ax1 ? 1.0 : 0.0, e2 = (!ax0 && !ax1) ? 1.0 : 0.0;
    double v0 = g1 * e2 - g2 * e1, v1 = g2 * e0 - g0 * e2, v2 = g0 * e1 - g1 * e0;
    double cn = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    if (!(cn > 0.0)) {
      v0 = 0.0; v1 = 0.0; v2 = 1.0;
      cn = 1.0;
    }
    r.n0 = v0 / cn; r.n1 = v1 / cn; r.n2 = v2 / cn;
  }
  r.lam = l * s;
  return r;
}

// normal_estimation.cpp:84-118: kNN(k) including the point itself, covariance,
// eigenvector of the smallest eigenvalue, curvature = |l0 / trace|, flipped so
// that (vp - p).n >= 0, optionally negated afterwards.  The covariance sums run
// in FP32 over offsets from the query point, in the order the unordered k-NN
// set reduction meets the neighbours; the eigen-solve is FP64.
// With a neighbour row (LCR_NORMALS_KEEP_NEIGHBOURS) it also records each
// neighbour's original index and the largest squared distance (NbrGraph).
struct NeAcc {
  float qx, qy, qz;
  const float4* __restrict__ xyz;
  float sx, sy, sz, sxx, sxy, sxz, syy, syz, szz;
  int m;
  uint32_t* row;
  float rmax;
  __device__ __forceinline__ void init(float x, float y, float z, const float4* p, uint32_t* r = nullptr) {
    qx = x; qy = y; qz = z;
    xyz = p;
    sx = sy = sz = sxx = sxy = sxz = syy = syz = szz = 0.f;
    m = 0;
    row = r;
    rmax = 0.f;
  }
  __device__ __forceinline__ void take(const float4& p) {
    const float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
    sx += dx; sy += dy; sz += dz;
    sxx += dx * dx; sxy += dx * dy; sxz += dx * dz;
    syy += dy * dy; syz += dy * dz; szz += dz * dz;
    ++m;
  }
  // p: a staged index point (w = original index), d its squared distance.
  // The k-set hands over exactly K <= kGraphMaxK points; the row write is
  // bounded all the same, so that no error upstream can write past a row.
  __device__ __forceinline__ void add(const float4& p, float d) {
    if (row && m < kGraphR) {
      row[m] = __float_as_uint(p.w);
      rmax = fmaxf(rmax, d);
    }
    take(p);
  }
  __device__ __forceinline__ void begin(float, int) {}
  __device__ __forceinline__ void add_key(unsigned long long k) {
    if (row && m < kGraphR) {
      row[m] = key_idx(k);
      rmax = fmaxf(rmax, key_dist(k));
    }
    take(xyz[key_idx(k)]);
  }
  // The row's radius word, once every neighbour is in (K asked for).
  __device__ __forceinline__ void finish_row(int K) {
    if (row) row[kGraphR] = __float_as_uint(m < K ? LCR_INF : rmax);
  }
};

__device__ __forceinline__ uint32_t* graph_row(uint32_t* rows, bool qv, float w) {
  return rows && qv ? rows + static_cast<size_t>(__float_as_uint(w)) * 32 : nullptr;
}

__device__ __forceinline__ void normal_store(const NeAcc& a, float vx, float vy, float vz, int flip_all, uint32_t o,
                                             float4* __restrict__ onrm) {
  const float nan = __int_as_float(0x7fc00000);
  if (a.m < 3) {
    onrm[o] = make_float4(nan, nan, nan, nan);
    return;
  }
  const double im = 1.0 / a.m;
  const double mx = a.sx * im, my = a.sy * im, mz = a.sz * im;
  const double C0 = a.sxx * im - mx * mx, C1 = a.sxy * im - mx * my, C2 = a.sxz * im - mx * mz,
               C3 = a.syy * im - my * my, C4 = a.syz * im - my * mz, C5 = a.szz * im - mz * mz;
  const Eig3 e = smallest_eig(C0, C1, C2, C3, C4, C5);
  const double tr = C0 + C3 + C5;
  const double curv = tr != 0.0 ? fabs(e.lam / tr) : 0.0;
  const double cs = static_cast<double>(__fsub_rn(vx, a.qx)) * e.n0 + static_cast<double>(__fsub_rn(vy, a.qy)) * e.n1 +
                    static_cast<double>(__fsub_rn(vz, a.qz)) * e.n2;
  double sgn = cs < 0 ? -1.0 : 1.0;
  if (flip_all) sgn = -sgn;
  onrm[o] = make_float4(static_cast<float>(sgn * e.n0), static_cast<float>(sgn * e.n1),
                        static_cast<float>(sgn * e.n2), static_cast<float>(curv));
}

__global__ void k_normals(IndexView ix, int K, const float4* __restrict__ xyz, float vx, float vy, float vz,
                          int flip_all, float4* __restrict__ onrm, EscapeQueue eq, uint32_t* __restrict__ rows) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wbase = smem + wib * kset_warp_bytes();
  const int tile = blockIdx.x * nw + wib;
  if (tile >= ix.nleaf) return;
  const float4 q = ix.pts[static_cast<size_t>(tile) * 32 + lane];
  const bool qv = finite3(q.x, q.y, q.z);
  float4 tlo, thi;
  if (!tile_box(q.x, q.y, q.z, qv, tlo, thi)) return;
  NeAcc acc;
  acc.init(q.x, q.y, q.z, xyz, graph_row(rows, qv, q.w));
  bool esc = false;
  float top = 0.f;
  tile_kset(ix, q.x, q.y, q.z, qv, K, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), wbase + sizeof(KnnWarp), tile,
            acc, 0.f, &esc, &top);
  if (esc) {
    escape_push(eq, static_cast<uint32_t>(tile) * 32u + lane, top);
  } else if (qv) {
    normal_store(acc, vx, vy, vz, flip_all, __float_as_uint(q.w), onrm);
    acc.finish_row(K);
  }
}

// One warp per escaped query (warps stride over the queue): the query alone
// as the tile, seeded with its own leaf and two either side, its histogram
// topped at four times the largest squared distance it met (an octave of
// distance above its k-th, so the k-th lies inside the range).
__global__ void k_normals_escaped(IndexView ix, int K, const float4* __restrict__ xyz, float vx, float vy, float vz,
                                  int flip_all, float4* __restrict__ onrm, EscapeQueue eq,
                                  uint32_t* __restrict__ rows) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wbase = smem + wib * kset_warp_bytes();
  const unsigned count = *eq.n;
  for (unsigned w = blockIdx.x * nw + wib; w < count; w += gridDim.x * nw) {
    const uint32_t slot = eq.slot[w];
    const float4 p = ix.pts[slot];
    const bool qv = lane == 0;
    const float qx = qv ? p.x : 0.f, qy = qv ? p.y : 0.f, qz = qv ? p.z : 0.f;
    float4 tlo, thi;
    tile_box(qx, qy, qz, qv, tlo, thi);
    NeAcc acc;
    acc.init(qx, qy, qz, xyz, graph_row(rows, qv, p.w));
    tile_kset(ix, qx, qy, qz, qv, K, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), wbase + sizeof(KnnWarp),
              static_cast<int>(slot >> 5), acc, 4.f * fmaxf(eq.top[w], 1e-30f));
    if (qv) {
      normal_store(acc, vx, vy, vz, flip_all, __float_as_uint(p.w), onrm);
      acc.finish_row(K);
    }
    __syncwarp();
  }
}

// Normals of SOR inliers from SOR's neighbour lists (no search).  A warp takes
// 32 inliers; for each, its source's list (K <= 64 unordered keys, two per
// lane) is masked to the inliers and bitonic-sorted across the warp, and the
// first k inlier keys -- the exact k nearest inliers when the list holds at
// least k of them -- give the covariance (FP32 sums over the warp, fixed
// shuffle tree); then every lane solves its own point's eigenproblem.  A point
// whose list holds fewer than k inliers is queued for k_normals_queued.
__device__ __forceinline__ void cswap(unsigned long long& x, unsigned long long u, bool keep_min) {
  x = keep_min ? (u < x ? u : x) : (u > x ? u : x);
}

__global__ void __launch_bounds__(256) k_normals_list(const unsigned long long* __restrict__ keys, int K,
                                                      const uint8_t* __restrict__ keep,
                                                      const uint32_t* __restrict__ rank,
                                                      const uint32_t* __restrict__ kept, int n, int k,
                                                      const float4* __restrict__ xyz, float vx, float vy, float vz,
                                                      int flip_all, float4* __restrict__ onrm,
                                                      uint32_t* __restrict__ queue, unsigned int* nqueue) {
  const int lane = threadIdx.x & 31;
  const int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
  if (base >= n) return;
  const unsigned long long none = ~0ull;
  NeAcc mine;
  mine.init(0.f, 0.f, 0.f, xyz);
  bool have = false;
  const int cnt_pts = min(32, n - base);
  // the lists of the warp's points are read one point ahead
  unsigned long long na = none, nb = none;
  float4 nq = make_float4(0.f, 0.f, 0.f, 0.f);
  auto fetch = [&](int j) {
    nq = xyz[base + j];
    na = nb = none;
    if (finite3(nq.x, nq.y, nq.z)) {
      const size_t o = kept[base + j];
      if (lane < K) na = keys[o * K + lane];
      if (lane + 32 < K) nb = keys[o * K + lane + 32];
    }
  };
  fetch(0);
  for (int j = 0; j < cnt_pts; ++j) {
    const float4 q = nq;
    unsigned long long a = na, b = nb;
    if (j + 1 < cnt_pts) fetch(j + 1);
    if (!finite3(q.x, q.y, q.z)) continue;  // not searched: stays NaN
    if (a != none && !keep[key_idx(a)]) a = none;
    if (b != none && !keep[key_idx(b)]) b = none;
    const int inl = __popc(__ballot_sync(LCR_FULL, a != none)) + __popc(__ballot_sync(LCR_FULL, b != none));
    if (inl < k) {
      if (lane == 0) queue[atomicAdd(nqueue, 1u)] = static_cast<uint32_t>(base + j);
      continue;
    }
    // ascending bitonic sort of the 64 keys: element lane in a, lane+32 in b
#pragma unroll
    for (int w = 2; w <= 64; w <<= 1) {
#pragma unroll
      for (int st = w >> 1; st > 0; st >>= 1) {
        if (st == 32) {
          const unsigned long long lo = a < b ? a : b, hi = a < b ? b : a;
          a = lo;
          b = hi;
        } else {
          const bool lower = (lane & st) == 0;
          const unsigned long long ua = __shfl_xor_sync(LCR_FULL, a, st);
          cswap(a, ua, lower == ((lane & w) == 0));
          const unsigned long long ub = __shfl_xor_sync(LCR_FULL, b, st);
          cswap(b, ub, lower == (((lane + 32) & w) == 0));
        }
      }
    }
    // covariance over the first k: elements lane (< k) and lane + 32 (< k)
    float t[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (lane < k) {
      const float4 p = xyz[rank[key_idx(a)]];
      const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
      t[0] = dx; t[1] = dy; t[2] = dz;
      t[3] = dx * dx; t[4] = dx * dy; t[5] = dx * dz; t[6] = dy * dy; t[7] = dy * dz; t[8] = dz * dz;
    }
    if (lane + 32 < k) {
      const float4 p = xyz[rank[key_idx(b)]];
      const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
      t[0] += dx; t[1] += dy; t[2] += dz;
      t[3] += dx * dx; t[4] += dx * dy; t[5] += dx * dz; t[6] += dy * dy; t[7] += dy * dz; t[8] += dz * dz;
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) t[c] = warp_sum(t[c]);
    if (lane == j) {
      mine.qx = q.x; mine.qy = q.y; mine.qz = q.z;
      mine.sx = t[0]; mine.sy = t[1]; mine.sz = t[2];
      mine.sxx = t[3]; mine.sxy = t[4]; mine.sxz = t[5]; mine.syy = t[6]; mine.syz = t[7]; mine.szz = t[8];
      mine.m = k;
      have = true;
    }
  }
  if (have) normal_store(mine, vx, vy, vz, flip_all, static_cast<uint32_t>(base + lane), onrm);
}

// Position of every point in the index's sorted order.
__global__ void k_index_pos(IndexView ix, uint32_t* __restrict__ pos) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ix.nleaf * 32) return;
  const uint32_t w = __float_as_uint(ix.pts[s].w);
  if (w != 0xffffffffu) pos[w] = static_cast<uint32_t>(s);
}

// Queued points (their list held fewer than k inliers): one warp per point, a
// search with that point as the tile's only query, seeded with its own leaf
// and two either side; its histogram range is set from its list's farthest
// entry (the k-th inlier lies beyond it).
__global__ void k_normals_queued(IndexView ix, int K, const float4* __restrict__ xyz, float vx, float vy, float vz,
                                 int flip_all, float4* __restrict__ onrm, const uint32_t* __restrict__ queue,
                                 const unsigned int* nqueue, const unsigned long long* __restrict__ keys, int LK,
                                 const uint32_t* __restrict__ kept, const uint32_t* __restrict__ pos) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wbase = smem + wib * kset_warp_bytes();
  const unsigned count = *nqueue;
  for (unsigned w = blockIdx.x * nw + wib; w < count; w += gridDim.x * nw) {
    const uint32_t i = queue[w];
    const float4 p = xyz[i];
    const size_t o = kept[i];
    float far2 = 0.f;
    for (int j = lane; j < LK; j += 32) far2 = fmaxf(far2, key_dist(keys[o * LK + j]));
    far2 = warp_max(far2);
    const bool qv = lane == 0;
    const float qx = qv ? p.x : 0.f, qy = qv ? p.y : 0.f, qz = qv ? p.z : 0.f;
    float4 tlo, thi;
    tile_box(qx, qy, qz, qv, tlo, thi);
    NeAcc acc;
    acc.init(qx, qy, qz, xyz);
    tile_kset(ix, qx, qy, qz, qv, K, tlo, thi, *reinterpret_cast<KnnWarp*>(wbase), wbase + sizeof(KnnWarp),
              static_cast<int>(pos[i] >> 5), acc, 256.f * fmaxf(far2, 1e-30f));
    if (qv) normal_store(acc, vx, vy, vz, flip_all, i, onrm);
    __syncwarp();
  }
}

// ----------------------------------------------------------------- crop
// accumulate_clouds.cpp:100-111: a source point p is redundant when some target
// q has float(q - r) <= p <= float(q + r) on every axis (the CropBox bounds are
// Vector4f(q.x - radius, ...) with a double radius).  Node test: for any member
// q of a box, float(q - r) >= float(lo - r) and float(q + r) <= float(hi + r).
struct Crop {
  float qx, qy, qz;
  bool qv, found, all;
  float4 tlo, thi;
  double r;
  __device__ __forceinline__ float lo_r(float v) const { return __double2float_rn(__dsub_rn(static_cast<double>(v), r)); }
  __device__ __forceinline__ float hi_r(float v) const { return __double2float_rn(__dadd_rn(static_cast<double>(v), r)); }
  __device__ __forceinline__ float metric(const float4& lo, const float4& hi) const {
    const bool hit = lo_r(lo.x) <= thi.x && hi_r(hi.x) >= tlo.x && lo_r(lo.y) <= thi.y && hi_r(hi.y) >= tlo.y &&
                     lo_r(lo.z) <= thi.z && hi_r(hi.z) >= tlo.z;
    return hit ? 0.f : LCR_INF;
  }
  __device__ __forceinline__ bool still(float m) const { return m <= 0.f && !all; }
  __device__ __forceinline__ bool need(const float4& lo, const float4& hi) const {
    return qv && !found && lo_r(lo.x) <= qx && qx <= hi_r(hi.x) && lo_r(lo.y) <= qy && qy <= hi_r(hi.y) &&
           lo_r(lo.z) <= qz && qz <= hi_r(hi.z);
  }
  __device__ __forceinline__ void scan(const float4* st) {
    for (int j = 0; j < 32 && !found; ++j) {
      const float4 t = st[j];
      if (qx >= lo_r(t.x) && qx <= hi_r(t.x) && qy >= lo_r(t.y) && qy <= hi_r(t.y) && qz >= lo_r(t.z) &&
          qz <= hi_r(t.z))
        found = true;
    }
  }
  __device__ __forceinline__ bool skip(int) const { return false; }
  __device__ __forceinline__ void visited(int) {}
  __device__ __forceinline__ void refresh() { all = __all_sync(LCR_FULL, !qv || found); }
};

__global__ void k_crop(IndexView tgt, IndexView src, double r, uint8_t* __restrict__ removed) {
  __shared__ WarpScratch wss[8];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x * (blockDim.x >> 5) + wib;
  if (tile >= src.nleaf) return;
  const float4 p = src.pts[static_cast<size_t>(tile) * 32 + lane];
  const bool qv = finite3(p.x, p.y, p.z);
  float4 tlo, thi;
  if (!tile_box(p.x, p.y, p.z, qv, tlo, thi)) return;
  Crop v;
  v.qx = p.x; v.qy = p.y; v.qz = p.z;
  v.qv = qv;
  v.found = false;
  v.tlo = tlo;
  v.thi = thi;
  v.r = r;
  v.refresh();
  tile_traverse(tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), wss[wib]);
  if (qv && v.found) removed[__float_as_uint(p.w)] = 1;
}

// PCL's CropBox (accumulate_clouds.cpp:103-110, negative mode) drops a source
// point that is not finite, and a box built on a non-finite target point holds
// every source point: each comparison with a NaN bound is false, so no point
// tests as outside it.  Pass 1 flags a non-finite target point; pass 2 starts
// the removed flags from that and from the source point's own finiteness.
__global__ void k_any_nonfinite(const float4* __restrict__ p, size_t n, int* __restrict__ flag) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool bad = i < n && !finite3(p[i].x, p[i].y, p[i].z);
  if (__any_sync(LCR_FULL, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void k_crop_init(const float4* __restrict__ src, size_t n, const int* __restrict__ tgt_bad,
                            uint8_t* __restrict__ removed) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  removed[i] = (*tgt_bad || !finite3(src[i].x, src[i].y, src[i].z)) ? 1 : 0;
}

size_t list_smem(int nw, int K) { return nw * knn_warp_bytes(K); }

constexpr int kListMaxK = 64;  // neighbour lists handed to the inliers hold at most this many keys

inline size_t align_up(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

__global__ void k_rank_of(const uint32_t* __restrict__ kept, int nkeep, uint32_t* __restrict__ rank) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nkeep) rank[kept[j]] = static_cast<uint32_t>(j);
}

// Warps per block of the unordered k-NN kernels come from ctx->tune (11 KB of
// shared memory per warp; the default 5 warps x 4 blocks = 20 resident warps
// per SM).  Every per-query result is independent of the block shape.

// Queue of tiles the unordered form hands to the sorted form: [0] = count,
// [1..] = tile ids.  Its grid: one block per SM, warps striding the queue.
struct RedoQueue {
  uint32_t* block;
  unsigned int* count() const { return reinterpret_cast<unsigned int*>(block); }
  uint32_t* tiles() const { return block + 1; }
};

RedoQueue redo_queue(lcr_ctx* ctx, int nleaf) {
  RedoQueue q;
  q.block = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * (static_cast<size_t>(nleaf) + 1)));
  CUDA_TRY(cudaMemsetAsync(q.block, 0, sizeof(uint32_t), ctx->stream));
  return q;
}


}  // namespace

void sor_run(lcr_ctx* ctx, const lcr_cloud* in, int mean_k, double std_mul, lcr_cloud** inliers,
             lcr_cloud** outliers, lcr_sor_stats* stats, float* host_dist) {
  if (mean_k <= 0) LCR_THROW(LCR_ERR_INVALID_ARG, "mean_k must be positive");
  const int n = static_cast<int>(in->n);
  if (n == 0) LCR_THROW(LCR_ERR_EMPTY, "statistical outlier removal on an empty cloud");
  const IndexView ix = cloud_index(ctx, in).v;
  const int K = mean_k + 1;
  const int nw = K <= 64 ? 4 : 2;
  const size_t smem = list_smem(nw, K);
  if (smem > 227 * 1024) LCR_THROW(LCR_ERR_INVALID_ARG, "mean_k=%d too large", mean_k);
  const int set_warps = ctx->tune.sor_warps;
  const size_t smem_set = set_warps * kset_warp_bytes();
  float* dist = static_cast<float*>(dev_alloc(ctx, sizeof(float) * n));
  uint8_t* flags = static_cast<uint8_t*>(dev_alloc(ctx, 3 * static_cast<size_t>(n)));
  uint8_t* valid = flags, *keep = flags + n, *drop = flags + 2 * static_cast<size_t>(n);
  const int nc0 = (n + 255) / 256;
  double* sums = static_cast<double*>(dev_alloc(ctx, sizeof(double) * (4 * static_cast<size_t>(nc0) + 8)));
  unsigned int* nvalid = reinterpret_cast<unsigned int*>(sums + 4 * nc0 + 4);
  int* too_few = reinterpret_cast<int*>(nvalid + 1);
  double* st = sums + 4 * nc0;
  CUDA_TRY(cudaMemsetAsync(dist, 0, sizeof(float) * n, ctx->stream));
  CUDA_TRY(cudaMemsetAsync(valid, 0, n, ctx->stream));
  CUDA_TRY(cudaMemsetAsync(sums + 4 * nc0 + 4, 0, 2 * sizeof(double), ctx->stream));
  const RedoQueue rq = redo_queue(ctx, ix.nleaf);
  char* eblk = static_cast<char*>(dev_alloc(ctx, 2 * align_up(sizeof(uint32_t) * n) + 256));
  EscapeQueue eq{reinterpret_cast<uint32_t*>(eblk), reinterpret_cast<float*>(eblk + align_up(sizeof(uint32_t) * n)),
                 reinterpret_cast<unsigned int*>(eblk + 2 * align_up(sizeof(uint32_t) * n))};
  CUDA_TRY(cudaMemsetAsync(eq.n, 0, sizeof(unsigned int), ctx->stream));
  // neighbour lists for the inliers' normals (k <= 64 only: two keys per lane there)
  NbrHint* hint = nullptr;
  unsigned long long* lists = nullptr;
  if (inliers && K <= kListMaxK) {
    hint = new NbrHint();
    const size_t b_keys = align_up(sizeof(unsigned long long) * K * static_cast<size_t>(n)),
                 b_keep = align_up(static_cast<size_t>(n)), b_rank = align_up(sizeof(uint32_t) * n);
    char* blk = static_cast<char*>(dev_alloc(ctx, b_keys + b_keep + 2 * b_rank));
    hint->block = blk;
    lists = reinterpret_cast<unsigned long long*>(blk);
    hint->keys = lists;
    hint->keep = reinterpret_cast<uint8_t*>(blk + b_keys);
    hint->rank = reinterpret_cast<uint32_t*>(blk + b_keys + b_keep);
    hint->kept = reinterpret_cast<uint32_t*>(blk + b_keys + b_keep + b_rank);
    hint->K = K;
    hint->n_src = n;
  }
  CUDA_TRY(cudaFuncSetAttribute(k_sor_dist, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_set)));
  CUDA_TRY(cudaFuncSetAttribute(k_sor_dist_sorted, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)));
  CUDA_TRY(cudaFuncSetAttribute(k_sor_dist_escaped, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem)));
  {
    KernelTimer kt(ctx, LCR_KT_SOR_KNN);
    LCR_LAUNCH(ctx, k_sor_dist, (ix.nleaf + set_warps - 1) / set_warps, set_warps * 32, smem_set, ix, mean_k, dist,
               valid, nvalid, rq.tiles(), rq.count(), too_few, lists, eq);
    LCR_LAUNCH(ctx, k_sor_dist_escaped, ctx->sms, nw * 32, smem, ix, mean_k, dist, valid, nvalid, lists, eq);
  }
  LCR_LAUNCH(ctx, k_sor_dist_sorted, ctx->sms, nw * 32, smem, ix, mean_k, dist, valid, nvalid, rq.tiles(), rq.count(),
             lists);
  dev_free(ctx, rq.block);
  dev_free(ctx, eblk);
  // blocked sums (ping-pong between two halves of `sums`)
  double *a = sums, *b = sums + nc0, *a2 = sums + 2 * nc0, *b2 = sums + 3 * nc0;
  int m = nc0;
  LCR_LAUNCH(ctx, k_bsum_level0, (m + 7) / 8, 256, 0, dist, n, a, b);  // a warp per chunk
  while (m > 1) {
    const int m2 = (m + 255) / 256;
    LCR_LAUNCH(ctx, k_bsum_level, (m2 + 7) / 8, 256, 0, a, b, m, a2, b2);
    std::swap(a, a2);
    std::swap(b, b2);
    m = m2;
  }
  LCR_LAUNCH(ctx, k_sor_threshold, 1, 32, 0, a, b, nvalid, std_mul, st);
  LCR_LAUNCH(ctx, k_sor_flags, (n + 255) / 256, 256, 0, dist, n, st, keep, drop);
  uint32_t* idx = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * n));
  // nvalid and too_few are adjacent: one copy
  unsigned int* h_chk = reinterpret_cast<unsigned int*>(static_cast<char*>(pinned(ctx, 64)) + 48);
  CUDA_TRY(cudaMemcpyAsync(h_chk, nvalid, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
  const int nkeep = compact_flags(ctx, keep, n, idx);  // synchronises
  if (h_chk[0] == 0 || h_chk[1] != 0) {
    dev_free(ctx, dist);
    dev_free(ctx, flags);
    dev_free(ctx, sums);
    dev_free(ctx, idx);
    if (hint) {
      dev_free(ctx, hint->block);
      delete hint;
    }
    LCR_THROW(LCR_ERR_TOO_FEW_POINTS, "SOR needs more than %d finite points (k+1 neighbours)", mean_k);
  }
  if (inliers) {
    *inliers = cloud_alloc(ctx, nkeep);
    gather_cloud(ctx, in, idx, nkeep, *inliers);
    // the inliers keep the input's sorted order: their index is a compaction
    if (nkeep > 0) (*inliers)->index = subset_index(ctx, *in->index, keep, idx, nkeep);
    if (hint && nkeep > 0) {
      CUDA_TRY(cudaMemcpyAsync(const_cast<uint8_t*>(hint->keep), keep, n, cudaMemcpyDeviceToDevice, ctx->stream));
      CUDA_TRY(cudaMemcpyAsync(const_cast<uint32_t*>(hint->kept), idx, sizeof(uint32_t) * nkeep,
                               cudaMemcpyDeviceToDevice, ctx->stream));
      LCR_LAUNCH(ctx, k_rank_of, (nkeep + 255) / 256, 256, 0, hint->kept, nkeep, const_cast<uint32_t*>(hint->rank));
      (*inliers)->nbr = hint;
      hint = nullptr;
    }
  }
  if (hint) {
    dev_free(ctx, hint->block);
    delete hint;
  }
  if (outliers) {
    const int ndrop = compact_flags(ctx, drop, n, idx);
    *outliers = cloud_alloc(ctx, ndrop);
    gather_cloud(ctx, in, idx, ndrop, *outliers);
  }
  double* hs = static_cast<double*>(pinned(ctx, 64));
  CUDA_TRY(cudaMemcpyAsync(hs, st, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(hs + 4, nvalid, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
  if (host_dist) CUDA_TRY(cudaMemcpyAsync(host_dist, dist, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  if (stats) {
    stats->mean = hs[0];
    stats->stddev = hs[1];
    stats->threshold = hs[2];
    stats->valid = *reinterpret_cast<unsigned int*>(hs + 4);
    stats->kept = static_cast<size_t>(nkeep);
    stats->removed = static_cast<size_t>(n - nkeep);
  }
  dev_free(ctx, dist);
  dev_free(ctx, flags);
  dev_free(ctx, sums);
  dev_free(ctx, idx);
}

lcr_cloud* normals_run(lcr_ctx* ctx, const lcr_cloud* in, int k, const float vp[3], int flags) {
  if (k <= 0) LCR_THROW(LCR_ERR_INVALID_ARG, "k must be positive");
  const int n = static_cast<int>(in->n);
  lcr_cloud* out = cloud_alloc(ctx, n);
  if (n == 0) return out;
  const IndexView ix = cloud_index(ctx, in).v;
  CUDA_TRY(cudaMemcpyAsync(out->xyz, in->xyz, sizeof(float4) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(out->rgb, in->rgb, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  // non-finite points keep NaN normals (they are not searched)
  CUDA_TRY(cudaMemsetAsync(out->nrm, 0xff, sizeof(float4) * n, ctx->stream));
  const int set_warps = ctx->tune.ne_warps;
  const size_t smem_set = set_warps * kset_warp_bytes();
  const int flip = (flags & LCR_NORMALS_FLIP_ALL) ? 1 : 0;
  // the neighbour rows come from the search below (the SOR-list path selects
  // from lists of another cloud's numbering and does not produce them)
  const bool keep = (flags & LCR_NORMALS_KEEP_NEIGHBOURS) != 0 && k <= kGraphMaxK;
  const NbrHint* h = in->nbr;
  if (!keep && h && k <= h->K && h->K <= kListMaxK) {
    // SOR inliers: select from SOR's neighbour lists; points whose list holds
    // fewer than k inliers are searched one per warp
    char* tmp = static_cast<char*>(dev_alloc(ctx, 2 * align_up(sizeof(uint32_t) * n) + 256));
    uint32_t* queue = reinterpret_cast<uint32_t*>(tmp);
    uint32_t* pos = reinterpret_cast<uint32_t*>(tmp + align_up(sizeof(uint32_t) * n));
    unsigned int* nq = reinterpret_cast<unsigned int*>(tmp + 2 * align_up(sizeof(uint32_t) * n));
    CUDA_TRY(cudaMemsetAsync(nq, 0, sizeof(unsigned int), ctx->stream));
    {
      KernelTimer kt(ctx, LCR_KT_NORMALS_KNN);
      LCR_LAUNCH(ctx, k_normals_list, (n + 255) / 256, 256, 0, h->keys, h->K, h->keep, h->rank, h->kept, n, k,
                 in->xyz, vp[0], vp[1], vp[2], flip, out->nrm, queue, nq);
    }
    CUDA_TRY(cudaFuncSetAttribute(k_normals_queued, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(smem_set)));
    LCR_LAUNCH(ctx, k_index_pos, (ix.nleaf * 32 + 255) / 256, 256, 0, ix, pos);
    LCR_LAUNCH(ctx, k_normals_queued, ctx->sms * 2, set_warps * 32, smem_set, ix, k, in->xyz, vp[0], vp[1], vp[2],
               flip, out->nrm, queue, nq, h->keys, h->K, h->kept, pos);
    dev_free(ctx, tmp);
    // the lists (8 B x (k+1) per point) are released once consumed: a second
    // normals call on this cloud searches
    dev_free(ctx, h->block);
    delete h;
    const_cast<lcr_cloud*>(in)->nbr = nullptr;
    out->index = share_index(in->index);
    return out;
  }
  CUDA_TRY(cudaFuncSetAttribute(k_normals, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_set)));
  CUDA_TRY(cudaFuncSetAttribute(k_normals_escaped, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(smem_set)));
  char* eblk = static_cast<char*>(dev_alloc(ctx, 2 * align_up(sizeof(uint32_t) * n) + 256));
  EscapeQueue eq{reinterpret_cast<uint32_t*>(eblk), reinterpret_cast<float*>(eblk + align_up(sizeof(uint32_t) * n)),
                 reinterpret_cast<unsigned int*>(eblk + 2 * align_up(sizeof(uint32_t) * n))};
  CUDA_TRY(cudaMemsetAsync(eq.n, 0, sizeof(unsigned int), ctx->stream));
  uint32_t* rows = nullptr;
  if (keep) {
    rows = static_cast<uint32_t*>(dev_alloc(ctx, sizeof(uint32_t) * 32 * static_cast<size_t>(n)));
    out->graph = new NbrGraph;
    out->graph->rows = rows;
    out->graph->k = k;
  }
  {
    KernelTimer kt(ctx, LCR_KT_NORMALS_KNN);
    LCR_LAUNCH(ctx, k_normals, (ix.nleaf + set_warps - 1) / set_warps, set_warps * 32, smem_set, ix, k, in->xyz,
               vp[0], vp[1], vp[2], flip, out->nrm, eq, rows);
    LCR_LAUNCH(ctx, k_normals_escaped, ctx->sms, set_warps * 32, smem_set, ix, k, in->xyz, vp[0], vp[1], vp[2],
               flip, out->nrm, eq, rows);
  }
  dev_free(ctx, eblk);
  out->index = share_index(in->index);  // same points in the same order
  return out;
}

void crop_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, double radius, uint8_t* d_removed) {
  if (src->n == 0) return;
  if (tgt->n == 0) {  // no box at all: nothing is cropped, non-finite points included
    CUDA_TRY(cudaMemsetAsync(d_removed, 0, src->n, ctx->stream));
    return;
  }
  int* bad = static_cast<int*>(dev_alloc(ctx, 256));
  CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  LCR_LAUNCH(ctx, k_any_nonfinite, static_cast<unsigned>((tgt->n + 255) / 256), 256, 0, tgt->xyz, tgt->n, bad);
  LCR_LAUNCH(ctx, k_crop_init, static_cast<unsigned>((src->n + 255) / 256), 256, 0, src->xyz, src->n, bad, d_removed);
  dev_free(ctx, bad);
  const IndexView tv = cloud_index(ctx, tgt).v;
  const IndexView sv = cloud_index(ctx, src).v;
  LCR_LAUNCH(ctx, k_crop, (sv.nleaf + 7) / 8, 256, 0, tv, sv, radius, d_removed);
}
