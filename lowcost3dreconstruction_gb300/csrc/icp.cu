// pcl::IterativeClosestPoint on the GPU (pcl_tools/fine_registration.cpp:105-126),
// for one pair (lcr_icp) or for many pairs at once (lcr_icp_batch).
//
// All pairs of a call iterate together; a pair that has converged drops out.
// One round (one ICP iteration of every live pair) is five launches over work
// queues that span the pairs, so uneven cloud sizes share the GPU:
//  1. k_icp_search  warps take tiles of 32 Hilbert-sorted source points from the
//                   concatenated tile list of all pairs, transform them by their
//                   pair's FP32 transform, find each point's exact nearest target
//                   within the correspondence distance (one shared warp-tile
//                   traversal), form the per-correspondence terms in FP32 and
//                   reduce them across the warp with a transposing reduce-
//                   scatter into a per-tile row.  Tiles wider than four search
//                   radii are deferred.
//  2. k_icp_hard    one warp per point of a deferred tile (per-query pruning).
//  3. k_icp_wide    the term rows of the deferred tiles.
//  4. k_icp_reduce  fixed-order FP64 sums of chunks of 64 tile rows.
//  5. k_icp_solve   one block per pair: FP64 solve (3x3 SVD for point-to-point,
//                   6x6 LDL^T for point-to-plane), compose, re-orthonormalise,
//                   PCL's DefaultConvergenceCriteria; the last block to finish
//                   sets the loop condition (some pair still live).
// The rounds run as the body of a CUDA-graph WHILE node captured once per
// context (LCR_ICP_GRAPH=0 runs them from a host loop).  Every sum runs in a
// fixed order per pair, so a pair's result does not depend on scheduling or on
// the other pairs of the batch.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "search.cuh"

namespace {

constexpr int kIcpThreads = 256;
constexpr int kIcpWarps = kIcpThreads / 32;
constexpr int kChunkTiles = 64;  // tile rows per reduction chunk

// Per pair, written by the host (the centroid by the device).
struct IcpParams {
  IndexView tgt;
  const float4* src_pts;  // Hilbert-sorted source (the source index's points)
  const float4* tgt_nrm;  // target normals by original index
  const float4* tgt_xyz;  // target points by original index
  int src_ntiles;
  int tile0, chunk0;      // first global tile / chunk of this pair
  float cap;              // FP32 form of max_correspondence_distance^2
  float c[3];             // centre of the linear algebra: target centroid (float)
  int min_corr;
  int max_iter;
  double teps, feps;
  int stop_iter;          // 0: off
  double stop_mse;        // stop_rms^2
  const uint32_t* tgt_rows;  // the target's neighbour rows (NbrGraph), or null
  int tgt_k;
};

// Per pair, device-resident across rounds.
struct IcpState {
  double T[16];
  Xf Tf;
  double prev_mse, mse, fitness;
  int iter, done, converged, state, ncorr, launches;
};

// The call: pair arrays and the scratch of all pairs (global slot = global
// tile * 32 + lane).
struct BatchDesc {
  int npairs, total_tiles, total_chunks, use_graph;
  IcpParams* prm;
  IcpState* st;
  const int* tile0;       // [npairs + 1] prefix of source tiles
  const int* chunk0;      // [npairs + 1] prefix of reduction chunks
  float* tile_part;       // [total_tiles][32] FP32 term rows
  uint32_t* hard_q;       // deferred query global slots
  float4* hard_tp;        // per global slot: target xyz, distance of a deferred query
  uint32_t* hard_ti;      // per global slot: its target index (0xffffffff: none)
  uint32_t* wide_tiles;   // global tiles whose rows wait for the deferred queries
  double* red;            // [total_chunks][32] FP64 chunk sums
  float* fd;              // fitness: squared NN distance per global slot (< 0: not a point)
  float4* far;            // fitness: queries with no target inside the cap (w = global slot)
  uint32_t* prev_ti;      // per global slot: last round's correspondence (0xffffffff: none)
};

// Work-queue counters, reset by the last solve block of every round.
struct BatchCounters {
  unsigned int tile_ctr, nhard, hard_ctr, nwide, wide_ctr, chunk_ctr;
  unsigned int ticket, active, rounds, live;
  unsigned int fit_tile_ctr, nfar, far_ctr;
  int max_rounds;
};

// Transposing warp reduction: on entry every lane holds 32 terms; on exit lane l
// holds the sum over the warp of term l (31 shuffles instead of 32*5).
__device__ __forceinline__ float reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = (lane & s) != 0;
#pragma unroll
    for (int i = 0; i < s; ++i) {
      const float send = up ? v[i] : v[i + s];
      const float keep = up ? v[i + s] : v[i];
      v[i] = keep + __shfl_xor_sync(LCR_FULL, send, s);
    }
  }
  return v[0];
}

// ---------------------------------------------------------- FP64 solvers
__device__ void svd3_jacobi(const double A[9], double U[9], double sv[3], double V[9]) {
  double a[3][3];  // a[col][row]
  double v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};  // v[col][row]
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) a[c][r] = A[3 * r + c];
  for (int sweep = 0; sweep < 12; ++sweep) {
    double off = 0.0;
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const double al = a[p][0] * a[p][0] + a[p][1] * a[p][1] + a[p][2] * a[p][2];
      const double be = a[q][0] * a[q][0] + a[q][1] * a[q][1] + a[q][2] * a[q][2];
      const double ga = a[p][0] * a[q][0] + a[p][1] * a[q][1] + a[p][2] * a[q][2];
      const double nrm = sqrt(al * be);
      if (!(fabs(ga) > 1e-15 * nrm)) continue;
      off = fmax(off, fabs(ga) / nrm);
      const double zeta = (be - al) / (2.0 * ga);
      const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
      for (int i = 0; i < 3; ++i) {
        const double x = a[p][i], y = a[q][i];
        a[p][i] = cs * x - sn * y;
        a[q][i] = sn * x + cs * y;
        const double vx = v[p][i], vy = v[q][i];
        v[p][i] = cs * vx - sn * vy;
        v[q][i] = sn * vx + cs * vy;
      }
    }
    if (off < 1e-15) break;
  }
  double s[3];
  int ord[3] = {0, 1, 2};
  for (int c = 0; c < 3; ++c) s[c] = sqrt(a[c][0] * a[c][0] + a[c][1] * a[c][1] + a[c][2] * a[c][2]);
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2 - i; ++j)
      if (s[ord[j]] < s[ord[j + 1]]) {
        const int tmp = ord[j]; ord[j] = ord[j + 1]; ord[j + 1] = tmp;
      }
  double u[3][3];
  const double scale = s[ord[0]] > 0 ? s[ord[0]] : 1.0;
  for (int k = 0; k < 3; ++k) {
    const int c = ord[k];
    sv[k] = s[c];
    for (int r = 0; r < 3; ++r) V[3 * r + k] = v[c][r];
    if (s[c] > 1e-13 * scale) {
      for (int r = 0; r < 3; ++r) u[k][r] = a[c][r] / s[c];
    } else if (k == 2) {
      u[2][0] = u[0][1] * u[1][2] - u[0][2] * u[1][1];
      u[2][1] = u[0][2] * u[1][0] - u[0][0] * u[1][2];
      u[2][2] = u[0][0] * u[1][1] - u[0][1] * u[1][0];
    } else {
      // rank <= 1: complete with an axis orthogonal to the previous columns
      for (int tries = 0; tries < 3; ++tries) {
        double cand[3] = {tries == 0 ? 1.0 : 0.0, tries == 1 ? 1.0 : 0.0, tries == 2 ? 1.0 : 0.0};
        for (int pcol = 0; pcol < k; ++pcol) {
          const double d = cand[0] * u[pcol][0] + cand[1] * u[pcol][1] + cand[2] * u[pcol][2];
          for (int r = 0; r < 3; ++r) cand[r] -= d * u[pcol][r];
        }
        const double cn = sqrt(cand[0] * cand[0] + cand[1] * cand[1] + cand[2] * cand[2]);
        if (cn > 0.5) {
          for (int r = 0; r < 3; ++r) u[k][r] = cand[r] / cn;
          break;
        }
      }
    }
  }
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < 3; ++r) U[3 * r + k] = u[k][r];
}

__device__ double det3(const double M[9]) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
}

// SPD 6x6 solve by LDL^T; pivots below 1e-12 of the largest diagonal count as
// singular (degenerate correspondence geometry).
__device__ __forceinline__ bool ldlt6(const double M[36], const double b[6], double x[6]) {
  // fully unrolled: every index is a constant, so M, L, D stay in registers
  double L[36], D[6];
  double dmax = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) dmax = fmax(dmax, fabs(M[7 * i]));
  if (!(dmax > 0)) return false;
#pragma unroll
  for (int i = 0; i < 36; ++i) L[i] = 0;
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = M[6 * j + j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= L[6 * j + k] * L[6 * j + k] * D[k];
    ok = ok && d > 1e-12 * dmax;
    D[j] = d;
    L[6 * j + j] = 1.0;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double v = M[6 * i + j];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= L[6 * i + k] * L[6 * j + k] * D[k];
      L[6 * i + j] = v / d;
    }
  }
  if (!ok) return false;
  double y[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double v = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) v -= L[6 * i + k] * y[k];
    y[i] = v;
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) y[i] /= D[i];
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    double v = y[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) v -= L[6 * k + i] * x[k];
    x[i] = v;
  }
  return true;
}

// Point-to-point (Umeyama without scale): terms S[0..2] = sum s', S[3..5] = sum t',
// S[6+3a+b] = sum t'_a s'_b with s' = s - c, t' = t - c.
__device__ bool solve_point(const double* S, const double c[3], double n, double dT[16]) {
  double ms[3], mt[3], Sg[9];
  for (int a = 0; a < 3; ++a) { ms[a] = S[a] / n; mt[a] = S[3 + a] / n; }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) Sg[3 * a + b] = S[6 + 3 * a + b] / n - mt[a] * ms[b];
  double U[9], sv[3], V[9];
  svd3_jacobi(Sg, U, sv, V);
  const double D = (det3(U) * det3(V) < 0) ? -1.0 : 1.0;
  double R[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = U[3 * i] * V[3 * j] + U[3 * i + 1] * V[3 * j + 1] + D * U[3 * i + 2] * V[3 * j + 2];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) dT[4 * i + j] = R[3 * i + j];
    const double mti = mt[i] + c[i];
    dT[4 * i + 3] = mti - (R[3 * i] * (ms[0] + c[0]) + R[3 * i + 1] * (ms[1] + c[1]) + R[3 * i + 2] * (ms[2] + c[2]));
  }
  dT[12] = dT[13] = dT[14] = 0.0;
  dT[15] = 1.0;
  return true;
}

// Point-to-plane linear least squares about c: S[0..20] upper triangle of A^T A,
// S[21..26] A^T b, rows A = [ s' x n, n ], b = n.(t' - s').  R = Rz Ry Rx.
__device__ __forceinline__ bool solve_plane(const double* S, const double c[3], double dT[16]) {
  double M[36], b[6], x[6];
  int k = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      M[6 * i + j] = S[k];
      M[6 * j + i] = S[k];
      ++k;
    }
#pragma unroll
  for (int i = 0; i < 6; ++i) b[i] = S[21 + i];
  if (!ldlt6(M, b, x)) return false;
  double sa, ca, sb, cb, sg, cg;
  sincos(x[0], &sa, &ca);
  sincos(x[1], &sb, &cb);
  sincos(x[2], &sg, &cg);
  const double R[9] = {cg * cb, -sg * ca + cg * sb * sa, sg * sa + cg * sb * ca,
                       sg * cb, cg * ca + sg * sb * sa,  -cg * sa + sg * sb * ca,
                       -sb,     cb * sa,                 cb * ca};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) dT[4 * i + j] = R[3 * i + j];
    dT[4 * i + 3] = x[3 + i] + c[i] - (R[3 * i] * c[0] + R[3 * i + 1] * c[1] + R[3 * i + 2] * c[2]);
  }
  dT[12] = dT[13] = dT[14] = 0.0;
  dT[15] = 1.0;
  return true;
}

__device__ __forceinline__ void orthonormalize(double T[16]) {
  double r0[3] = {T[0], T[1], T[2]}, r1[3] = {T[4], T[5], T[6]};
  const double n0 = sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
  for (int i = 0; i < 3; ++i) r0[i] /= n0;
  const double d = r0[0] * r1[0] + r0[1] * r1[1] + r0[2] * r1[2];
  for (int i = 0; i < 3; ++i) r1[i] -= d * r0[i];
  const double n1 = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  for (int i = 0; i < 3; ++i) r1[i] /= n1;
  T[0] = r0[0]; T[1] = r0[1]; T[2] = r0[2];
  T[4] = r1[0]; T[5] = r1[1]; T[6] = r1[2];
  T[8] = r0[1] * r1[2] - r0[2] * r1[1];
  T[9] = r0[2] * r1[0] - r0[0] * r1[2];
  T[10] = r0[0] * r1[1] - r0[1] * r1[0];
}

// One ICP iteration's bookkeeping (PCL computeTransformation loop body with
// DefaultConvergenceCriteria as the reference tool configures it).
template <int P2PL>
__device__ __forceinline__ void icp_update(const double* S, const IcpParams* prm, IcpState* st) {
  const double cnt = P2PL ? S[27] : S[15];
  const double dsum = P2PL ? S[28] : S[16];
  const int ncorr = static_cast<int>(cnt + 0.5);
  st->ncorr = ncorr;
  if (ncorr < prm->min_corr) {
    st->converged = 0;
    st->state = LCR_ICP_STATE_NO_CORRESPONDENCES;
    st->done = 1;
    return;
  }
  const double mse = dsum / cnt;
  st->mse = mse;
  const double c[3] = {prm->c[0], prm->c[1], prm->c[2]};
  double dT[16];
  const bool ok = P2PL ? solve_plane(S, c, dT) : solve_point(S, c, ncorr, dT);
  if (!ok) {
    st->converged = 0;
    st->state = LCR_ICP_STATE_NO_CORRESPONDENCES;
    st->done = 1;
    return;
  }
  double T[16], T0[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) T0[i] = st->T[i];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double s = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) s += dT[4 * i + k] * T0[4 * k + j];
      T[4 * i + j] = s;
    }
  orthonormalize(T);
  for (int i = 0; i < 16; ++i) st->T[i] = T[i];
  for (int i = 0; i < 12; ++i) st->Tf.m[i] = static_cast<float>(T[i]);
  st->iter += 1;
  if (st->iter >= prm->max_iter) {
    st->converged = 1;
    st->state = LCR_ICP_STATE_ITERATIONS;
    st->done = 1;
    return;
  }
  // The increment is judged as PCL's Matrix4f: its float cast, read in double.
  const double f00 = static_cast<float>(dT[0]), f11 = static_cast<float>(dT[5]), f22 = static_cast<float>(dT[10]);
  const double f03 = static_cast<float>(dT[3]), f13 = static_cast<float>(dT[7]), f23 = static_cast<float>(dT[11]);
  const double cos_angle = 0.5 * (f00 + f11 + f22 - 1);
  const double tsq = f03 * f03 + f13 * f13 + f23 * f23;
  if (cos_angle >= 1.0 - prm->teps && tsq <= prm->teps) {
    st->converged = 1;
    st->state = LCR_ICP_STATE_TRANSFORM;
    st->done = 1;
    return;
  }
  const double dm = fabs(mse - st->prev_mse);
  if (dm < 1e-12) {
    st->converged = 1;
    st->state = LCR_ICP_STATE_ABS_MSE;
    st->done = 1;
    return;
  }
  if (dm / st->prev_mse < prm->feps) {
    st->converged = 1;
    st->state = LCR_ICP_STATE_REL_MSE;
    st->done = 1;
    return;
  }
  st->prev_mse = mse;
  if (prm->stop_iter > 0 && st->iter >= prm->stop_iter && mse > prm->stop_mse) {
    st->converged = 0;
    st->state = LCR_ICP_STATE_STOPPED;
    st->done = 1;
  }
}
// Terms of one correspondence (all zero when the source point has none):
// point-to-point S[0..2] s', S[3..5] t', S[6+3a+b] t'_a s'_b, S[15] count,
// S[16] distance; point-to-plane S[0..20] upper A^T A, S[21..26] A^T b,
// S[27] count, S[28] distance; s' = s - c, t' = t - c.
template <int P2PL>
__device__ __forceinline__ void corr_terms(float (&t)[32], bool found, const float3& q, const float4& tp, float d,
                                           uint32_t tidx, const IcpParams* __restrict__ prm) {
#pragma unroll
  for (int i = 0; i < 32; ++i) t[i] = 0.f;
  if (!found) return;
  const float c0 = prm->c[0], c1 = prm->c[1], c2 = prm->c[2];
  const float sx = q.x - c0, sy = q.y - c1, sz = q.z - c2;
  const float tx = tp.x - c0, ty = tp.y - c1, tz = tp.z - c2;
  if (!P2PL) {
    t[0] = sx; t[1] = sy; t[2] = sz;
    t[3] = tx; t[4] = ty; t[5] = tz;
    t[6] = tx * sx; t[7] = tx * sy; t[8] = tx * sz;
    t[9] = ty * sx; t[10] = ty * sy; t[11] = ty * sz;
    t[12] = tz * sx; t[13] = tz * sy; t[14] = tz * sz;
    t[15] = 1.f;
    t[16] = d;
  } else {
    const float4 n = prm->tgt_nrm[tidx];
    t[27] = 1.f;
    t[28] = d;
    if (finite3(n.x, n.y, n.z)) {
      float A[6];
      A[0] = sy * n.z - sz * n.y;
      A[1] = sz * n.x - sx * n.z;
      A[2] = sx * n.y - sy * n.x;
      A[3] = n.x; A[4] = n.y; A[5] = n.z;
      const float r = n.x * (tx - sx) + n.y * (ty - sy) + n.z * (tz - sz);
      int k = 0;
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) t[k++] = A[i] * A[j];
#pragma unroll
      for (int i = 0; i < 6; ++i) t[21 + i] = A[i] * r;
    }
  }
}

// Pair owning global tile g: the last p with tile0[p] <= g.
__device__ __forceinline__ int pair_of(const int* __restrict__ pre, int npairs, int g) {
  int lo = 0, hi = npairs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&pre[mid]) <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Per-warp cache of the pair being worked on: its target index view and
// FP32 transform in shared memory (reloaded when the warp moves to another pair).
struct PairCache {
  IndexView tgt;
  Xf T;
  int pair;
};

__device__ __forceinline__ void cache_pair(PairCache& pc, const BatchDesc* __restrict__ d, int p, int lane) {
  if (pc.pair == p) return;
  __syncwarp();
  if (lane == 0) {
    pc.tgt = d->prm[p].tgt;
    pc.T = d->st[p].Tf;
    pc.pair = p;
  }
  __syncwarp();
}

__device__ __forceinline__ unsigned vload(const unsigned* p) { return *reinterpret_cast<const volatile unsigned*>(p); }

// Last round's correspondence of a slot as a starting candidate for this
// round's search: key (distance under the current transform, index) if it is
// still within the cap, else "none".
// Also returns that correspondence's index (prev, 0xffffffff: none) and its
// squared distance under the current transform whatever the cap (dd).
__device__ __forceinline__ void prev_candidate(const BatchDesc* __restrict__ d, const IcpParams* __restrict__ prm,
                                               int gslot, bool pv, const float3& q, unsigned long long& key,
                                               float4& p, uint32_t& prev, float& dd) {
  key = ~0ull;
  p = make_float4(0.f, 0.f, 0.f, 0.f);
  dd = LCR_INF;
  prev = pv ? d->prev_ti[gslot] : 0xffffffffu;
  if (prev == 0xffffffffu) return;
  p = prm->tgt_xyz[prev];
  dd = exact_dist2(q.x, q.y, q.z, p.x, p.y, p.z);
  if (dd <= prm->cap) key = make_key(dd, prev);
  p.w = __uint_as_float(prev);
}

// The nearest of row `row`'s k points to q: min of the (distance, index) keys,
// uncapped.  Four indices, then their four points, are loaded before any is
// used (two memory latencies per four points rather than one per point);
// words past k hold no index and are replaced by the row's own point c (a
// valid index) and masked out.
__device__ __forceinline__ unsigned long long row_min(const uint32_t* __restrict__ row, int k, uint32_t c,
                                                      const float4* __restrict__ xyz, const float3& q) {
  unsigned long long b = ~0ull;
#pragma unroll 2
  for (int j0 = 0; j0 < 32; j0 += 4) {
    if (j0 < k) {
      const uint4 ta = __ldg(reinterpret_cast<const uint4*>(row + j0));
      uint32_t t[4] = {ta.x, ta.y, ta.z, ta.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) t[u] = j0 + u < k ? t[u] : c;
      float4 p[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) p[u] = __ldg(xyz + t[u]);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const unsigned long long key = make_key(exact_dist2(q.x, q.y, q.z, p[u].x, p[u].y, p[u].z), t[u]);
        b = key < b ? key : b;
      }
    }
  }
  return b;
}

// The capped nearest target of q proven from the target's neighbour rows,
// without a search.  c is a target point at squared distance dc from q, and
// R, its row's radius word, is the largest squared distance from c to the k
// points of its row, so every target point t outside the row has
// D(c, t) >= R.  In true distances |qt| >= |ct| - |qc|, so R > 4 dc puts every
// such t strictly farther from q than c whenever the three rounded squared
// distances are within a factor (1 +- 1e-5) of the true ones: each is five
// roundings of positive terms (within 5 ulps, 3e-7), and the 1e-30 floor keeps
// subnormal squares out of it (dc == 0: q and c agree to 1e-22 while every t
// outside lies at least 1e-15 from c).  The 4.0001 factor holds the margin.
// Then the nearest under the (distance, index) order lies in the row, c
// included, and the row's minimum, capped, is the exact answer.
// Starting from c = s (last round's correspondence): when the test fails but
// R >= dc (within a factor 4 of passing), the row's nearest point b, strictly
// closer in key order, is tried once more with its own row.  A lane further
// off goes to the search at once: a few rows would not settle it, and their
// scattered loads cost more than its share of the tile's traversal.  Returns
// true with best = the capped answer, or false with seed = the best key met,
// a valid first bound for the search.
__device__ __forceinline__ bool row_proves(float R, float dc) {
  return R > 4.0001f * dc && R >= 1e-30f && (dc == 0.f || dc >= 1e-30f);
}
__device__ __forceinline__ bool graph_nn(const IcpParams* __restrict__ prm, const float3& q, uint32_t s, float ds,
                                         unsigned long long& best, unsigned long long& seed) {
  const int k = prm->tgt_k;
  const unsigned long long none = make_key(prm->cap, 0xffffffffu);
  uint32_t c = s;
  float dc = ds;
  seed = make_key(dc, c);
  const uint32_t* __restrict__ row = prm->tgt_rows + static_cast<size_t>(c) * 32;
  float R = __uint_as_float(__ldg(row + kGraphR));
  if (!(row_proves(R, dc) || R >= dc)) return false;
  unsigned long long b = row_min(row, k, c, prm->tgt_xyz, q);
  if (row_proves(R, dc)) {
    best = b < none ? b : none;
    return true;
  }
  if (!(b < seed)) return false;  // no closer point in the row
  seed = b;
  c = key_idx(b);
  dc = key_dist(b);
  row = prm->tgt_rows + static_cast<size_t>(c) * 32;
  R = __uint_as_float(__ldg(row + kGraphR));
  if (!row_proves(R, dc)) return false;
  b = row_min(row, k, c, prm->tgt_xyz, q);
  best = b < none ? b : none;
  return true;
}

// 1. Tiles of the live pairs: compact ones searched and reduced to a row,
// wide ones deferred.
template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_search(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  __shared__ WarpScratch wss[kIcpWarps];
  __shared__ PairCache pcs[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (lane == 0) pcs[wib].pair = -1;
  __syncwarp();
  const int total = d->total_tiles, npairs = d->npairs;
  for (;;) {
    int g = 0;
    if (lane == 0) g = static_cast<int>(atomicAdd(&cnt->tile_ctr, 1u));
    g = __shfl_sync(LCR_FULL, g, 0);
    if (g >= total) break;
    const int p = pair_of(d->tile0, npairs, g);
    const IcpParams* __restrict__ prm = d->prm + p;
    if (d->st[p].done) continue;  // its rows are not read this round
    cache_pair(pcs[wib], d, p, lane);
    const int gslot = g * 32 + lane;
    const float4 pt = prm->src_pts[(g - prm->tile0) * 32 + lane];
    const bool pv = finite3(pt.x, pt.y, pt.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    if (pv) q = xf_apply(pcs[wib].T, pt.x, pt.y, pt.z);
    const float cap = prm->cap;
    unsigned long long sk;
    float4 sp;
    uint32_t prev;
    float ds;
    prev_candidate(d, prm, gslot, pv, q, sk, sp, prev, ds);
    // lanes whose correspondence follows from the target's neighbour rows
    unsigned long long best = make_key(cap, 0xffffffffu);
    bool settled = false;
    if (prm->tgt_rows != nullptr && prev != 0xffffffffu) {
      unsigned long long g;
      settled = graph_nn(prm, q, prev, ds, best, g);
      if (!settled && g < sk) sk = g;  // a closer first bound for the search
    }
    const bool sv = pv && !settled;  // still to search
    float4 tlo, thi;
    if (tile_box(q.x, q.y, q.z, sv, tlo, thi)) {
      const float dx = thi.x - tlo.x, dy = thi.y - tlo.y, dz = thi.z - tlo.z;
      if (dx * dx + dy * dy + dz * dz > 16.f * cap) {
        // the lanes still to search go one per warp; the settled ones leave
        // their results in the per-slot arrays for the tile's row
        const unsigned valid = __ballot_sync(LCR_FULL, sv);
        unsigned base = 0;
        if (lane == 0) {
          base = atomicAdd(&cnt->nhard, static_cast<unsigned>(__popc(valid)));
          d->wide_tiles[atomicAdd(&cnt->nwide, 1u)] = static_cast<uint32_t>(g);
        }
        base = __shfl_sync(LCR_FULL, base, 0);
        if (sv) d->hard_q[base + __popc(valid & ((1u << lane) - 1u))] = static_cast<uint32_t>(gslot);
        if (settled) {
          const uint32_t ti = key_idx(best);
          const float4 tp = ti != 0xffffffffu ? prm->tgt_xyz[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
          d->hard_tp[gslot] = make_float4(tp.x, tp.y, tp.z, key_dist(best));
          d->hard_ti[gslot] = ti;
          d->prev_ti[gslot] = ti;
        }
        continue;
      }
      NN1 v;
      v.init(q.x, q.y, q.z, sv, cap, wss[wib]);
      v.seed(sk);
      tile_traverse(pcs[wib].tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z),
                    wss[wib]);
      if (sv) best = v.best;
    }
    d->prev_ti[gslot] = key_idx(best);
    const bool found = pv && key_idx(best) != 0xffffffffu;
    const float4 tp = found ? prm->tgt_xyz[key_idx(best)] : make_float4(0.f, 0.f, 0.f, 0.f);
    float t[32];
    corr_terms<P2PL>(t, found, q, tp, key_dist(best), key_idx(best), prm);
    d->tile_part[gslot] = reduce_scatter32(t, lane);
  }
}

// 2. The deferred queries, one per warp (exact per-query pruning); results
// land in per-slot arrays.
__global__ void __launch_bounds__(kIcpThreads) k_icp_hard(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  __shared__ WarpScratch wss[kIcpWarps];
  __shared__ PairCache pcs[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (lane == 0) pcs[wib].pair = -1;
  __syncwarp();
  const unsigned nhard = vload(&cnt->nhard);
  for (;;) {
    unsigned i = 0;
    if (lane == 0) i = atomicAdd(&cnt->hard_ctr, 1u);
    i = __shfl_sync(LCR_FULL, i, 0);
    if (i >= nhard) break;
    const uint32_t gslot = d->hard_q[i];
    const int g = static_cast<int>(gslot >> 5);
    const int p = pair_of(d->tile0, d->npairs, g);
    const IcpParams* __restrict__ prm = d->prm + p;
    cache_pair(pcs[wib], d, p, lane);
    const float4 pt = prm->src_pts[(g - prm->tile0) * 32 + (gslot & 31u)];
    const float3 q = xf_apply(pcs[wib].T, pt.x, pt.y, pt.z);
    unsigned long long sk;
    float4 sp;
    uint32_t prev;
    float ds;
    prev_candidate(d, prm, static_cast<int>(gslot), true, q, sk, sp, prev, ds);
    unsigned long long best;
    float4 bp;
    warp_query_nn(pcs[wib].tgt, q.x, q.y, q.z, prm->cap, wss[wib], best, bp, sk, sp);
    if (lane == 0) {
      d->hard_tp[gslot] = make_float4(bp.x, bp.y, bp.z, key_dist(best));
      d->hard_ti[gslot] = key_idx(best);
      d->prev_ti[gslot] = key_idx(best);
    }
  }
}

// 3. Rows of the deferred tiles from the per-slot results.
template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_wide(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned nwide = vload(&cnt->nwide);
  for (;;) {
    unsigned i = 0;
    if (lane == 0) i = atomicAdd(&cnt->wide_ctr, 1u);
    i = __shfl_sync(LCR_FULL, i, 0);
    if (i >= nwide) break;
    const int g = static_cast<int>(d->wide_tiles[i]);
    const int p = pair_of(d->tile0, d->npairs, g);
    const IcpParams* __restrict__ prm = d->prm + p;
    const int gslot = g * 32 + lane;
    const float4 pt = prm->src_pts[(g - prm->tile0) * 32 + lane];
    const bool pv = finite3(pt.x, pt.y, pt.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    float4 tp = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t ti = 0xffffffffu;
    if (pv) {
      q = xf_apply(d->st[p].Tf, pt.x, pt.y, pt.z);
      tp = d->hard_tp[gslot];
      ti = d->hard_ti[gslot];
    }
    float t[32];
    corr_terms<P2PL>(t, pv && ti != 0xffffffffu, q, tp, tp.w, ti, prm);
    d->tile_part[gslot] = reduce_scatter32(t, lane);
  }
}

// 4. Fixed-order FP64 sums: chunk c of pair p covers its tiles
// [64 (c - chunk0[p]), +64); within a chunk warp w adds tiles w, w+8, ...
__global__ void __launch_bounds__(kIcpThreads) k_icp_reduce(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  __shared__ double s[kIcpWarps][32];
  const int term = threadIdx.x & 31, sub = threadIdx.x >> 5;
  for (int c = blockIdx.x; c < d->total_chunks; c += gridDim.x) {
    const int p = pair_of(d->chunk0, d->npairs, c);
    if (d->st[p].done) continue;
    const IcpParams* __restrict__ prm = d->prm + p;
    const int t0 = prm->tile0 + (c - prm->chunk0) * kChunkTiles;
    const int t1 = min(prm->tile0 + prm->src_ntiles, t0 + kChunkTiles);
    double acc = 0.0;
    for (int t = t0 + sub; t < t1; t += kIcpWarps) acc += static_cast<double>(d->tile_part[t * 32 + term]);
    s[sub][term] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
      double v = 0.0;
#pragma unroll
      for (int k = 0; k < kIcpWarps; ++k) v += s[k][threadIdx.x];
      d->red[static_cast<size_t>(c) * 32 + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

// 5. One block per live pair (blocks stride over the pairs): its chunk sums in
// order, the FP64 update; the last block to finish decides whether another
// round runs and resets the queues.
template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_solve(const BatchDesc* __restrict__ d, BatchCounters* cnt,
                                                           cudaGraphConditionalHandle h) {
  __shared__ double S[32];
  __shared__ double s_sl[kIcpWarps][32];
  __shared__ unsigned s_live;
  if (threadIdx.x == 0) s_live = 0;
  __syncthreads();
  for (int p = blockIdx.x; p < d->npairs; p += gridDim.x) {
    IcpState* st = d->st + p;
    if (st->done) continue;
    const IcpParams* __restrict__ prm = d->prm + p;
    {
      // chunk sums in a fixed order: slice k adds chunks k, k+8, ...; then the 8 slices
      const int term = threadIdx.x & 31, slice = threadIdx.x >> 5;
      const int c0 = prm->chunk0, c1 = d->chunk0[p + 1];
      double v = 0.0;
      for (int c = c0 + slice; c < c1; c += kIcpWarps) v += d->red[static_cast<size_t>(c) * 32 + term];
      s_sl[slice][term] = v;
      __syncthreads();
      if (threadIdx.x < 32) {
        double w = 0.0;
#pragma unroll
        for (int k = 0; k < kIcpWarps; ++k) w += s_sl[k][threadIdx.x];
        S[threadIdx.x] = w;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      icp_update<P2PL>(S, prm, st);
      st->launches += 1;
      if (st->launches > prm->max_iter + 1) st->done = 1;  // hard bound on the device loop
      if (!st->done) ++s_live;
    }
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  if (s_live) atomicAdd(&cnt->active, s_live);
  __threadfence();
  const unsigned ticket = atomicAdd(&cnt->ticket, 1u);
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  const unsigned live = vload(&cnt->active);
  const unsigned rounds = cnt->rounds + 1;
  cnt->rounds = rounds;
  cnt->live = live;
  cnt->tile_ctr = 0;
  cnt->nhard = 0;
  cnt->hard_ctr = 0;
  cnt->nwide = 0;
  cnt->wide_ctr = 0;
  cnt->active = 0;
  cnt->ticket = 0;
  if (d->use_graph) cudaGraphSetConditional(h, (live > 0 && static_cast<int>(rounds) < cnt->max_rounds) ? 1u : 0u);
}

// getFitnessScore(): mean squared distance from every transformed source point
// to its exact (uncapped) nearest target point.  Phase 1 searches the tiles
// with the correspondence cap (a far lane would otherwise widen its whole
// tile's search); lanes with no target inside the cap, and all points of a
// tile wider than four search radii, are queued, and phase 2 finds their
// nearest point with one warp per query.  Distances land in fd[] by global
// slot and are summed per pair in a fixed order.
__global__ void __launch_bounds__(kIcpThreads) k_fitness(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  __shared__ WarpScratch wss[kIcpWarps];
  __shared__ PairCache pcs[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (lane == 0) pcs[wib].pair = -1;
  __syncwarp();
  float* __restrict__ fd = d->fd;
  for (;;) {
    int g = 0;
    if (lane == 0) g = static_cast<int>(atomicAdd(&cnt->fit_tile_ctr, 1u));
    g = __shfl_sync(LCR_FULL, g, 0);
    if (g >= d->total_tiles) break;
    const int p = pair_of(d->tile0, d->npairs, g);
    const IcpParams* __restrict__ prm = d->prm + p;
    cache_pair(pcs[wib], d, p, lane);
    const int gslot = g * 32 + lane;
    const float4 pt = prm->src_pts[(g - prm->tile0) * 32 + lane];
    const bool pv = finite3(pt.x, pt.y, pt.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    if (pv) q = xf_apply(pcs[wib].T, pt.x, pt.y, pt.z);
    float4 tlo, thi;
    if (!tile_box(q.x, q.y, q.z, pv, tlo, thi)) {
      fd[gslot] = -1.f;
      continue;
    }
    const float dx = thi.x - tlo.x, dy = thi.y - tlo.y, dz = thi.z - tlo.z;
    bool found = false;
    float dist = 0.f;
    if (!(dx * dx + dy * dy + dz * dz > 16.f * prm->cap)) {
      NN1 v;
      v.init(q.x, q.y, q.z, pv, prm->cap, wss[wib]);
      unsigned long long sk;
      float4 sp;
      uint32_t prev;
      float ds;
      prev_candidate(d, prm, gslot, pv, q, sk, sp, prev, ds);
      v.seed(sk);
      tile_traverse(pcs[wib].tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z),
                    wss[wib]);
      found = v.found();
      dist = key_dist(v.best);
    }
    if (!pv) {
      fd[gslot] = -1.f;  // not a point
    } else if (found) {
      fd[gslot] = dist;
    }
    // queue the rest, one reservation per warp
    const bool far = pv && !found;
    const unsigned m = __ballot_sync(LCR_FULL, far);
    unsigned base = 0;
    if (lane == 0 && m) base = atomicAdd(&cnt->nfar, static_cast<unsigned>(__popc(m)));
    base = __shfl_sync(LCR_FULL, base, 0);
    if (far) d->far[base + __popc(m & ((1u << lane) - 1u))] = make_float4(q.x, q.y, q.z, __int_as_float(gslot));
  }
}

__global__ void __launch_bounds__(kIcpThreads) k_fitness_far(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  __shared__ WarpScratch wss[kIcpWarps];
  __shared__ PairCache pcs[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (lane == 0) pcs[wib].pair = -1;
  __syncwarp();
  const unsigned nfar = vload(&cnt->nfar);
  constexpr unsigned kRun = 8;  // consecutive queue entries per grab: neighbours of one tile
  for (;;) {
    unsigned i0 = 0;
    if (lane == 0) i0 = atomicAdd(&cnt->far_ctr, kRun);
    i0 = __shfl_sync(LCR_FULL, i0, 0);
    if (i0 >= nfar) break;
    // each query starts from the previous query's nearest point (same pair):
    // an exact search with a near bound from the first node on
    unsigned long long prev_key = ~0ull;
    float4 prev_p = make_float4(0.f, 0.f, 0.f, 0.f);
    int prev_pair = -1;
    for (unsigned i = i0; i < min(nfar, i0 + kRun); ++i) {
      const float4 q = d->far[i];
      const int gslot = __float_as_int(q.w);
      const int p = pair_of(d->tile0, d->npairs, gslot >> 5);
      cache_pair(pcs[wib], d, p, lane);
      unsigned long long seed = ~0ull;
      if (p == prev_pair && prev_key != ~0ull)
        seed = make_key(exact_dist2(q.x, q.y, q.z, prev_p.x, prev_p.y, prev_p.z), key_idx(prev_key));
      unsigned long long best;
      float4 bp;
      warp_query_nn(pcs[wib].tgt, q.x, q.y, q.z, LCR_INF, wss[wib], best, bp, seed, prev_p);
      if (lane == 0) d->fd[gslot] = key_dist(best);
      prev_key = best;
      prev_p = bp;
      prev_pair = p;
    }
  }
}

// Per reduction chunk (64 tiles of one pair): sum and count of the valid
// distances, threads striding the chunk's slots, then a fixed tree; the chunk
// pairs (sum, count) land in red[] (reused: the rounds are over).
__global__ void __launch_bounds__(kIcpThreads) k_fitness_chunks(const BatchDesc* __restrict__ d) {
  __shared__ double s_s[kIcpWarps], s_c[kIcpWarps];
  for (int c = blockIdx.x; c < d->total_chunks; c += gridDim.x) {
    const int p = pair_of(d->chunk0, d->npairs, c);
    const IcpParams* __restrict__ prm = d->prm + p;
    const int t0 = prm->tile0 + (c - prm->chunk0) * kChunkTiles;
    const int t1 = min(prm->tile0 + prm->src_ntiles, t0 + kChunkTiles);
    double s = 0.0, n = 0.0;
    for (int i = t0 * 32 + static_cast<int>(threadIdx.x); i < t1 * 32; i += blockDim.x) {
      const float v = d->fd[i];
      if (v >= 0.f) {
        s += v;
        n += 1.0;
      }
    }
    s = warp_sum(s);
    n = warp_sum(n);
    if ((threadIdx.x & 31) == 0) {
      s_s[threadIdx.x >> 5] = s;
      s_c[threadIdx.x >> 5] = n;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double ts = 0.0, tc = 0.0;
      for (int w = 0; w < kIcpWarps; ++w) {
        ts += s_s[w];
        tc += s_c[w];
      }
      d->red[2 * static_cast<size_t>(c)] = ts;
      d->red[2 * static_cast<size_t>(c) + 1] = tc;
    }
    __syncthreads();
  }
}

// One warp per pair: its chunks in order (lane l adds chunks l, l+32, ...),
// then the fixed shuffle tree.
__global__ void __launch_bounds__(kIcpThreads) k_fitness_reduce(const BatchDesc* __restrict__ d, BatchCounters* cnt) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int p = warp; p < d->npairs; p += nwarps) {
    double s = 0.0, n = 0.0;
    for (int c = d->prm[p].chunk0 + lane; c < d->chunk0[p + 1]; c += 32) {
      s += d->red[2 * static_cast<size_t>(c)];
      n += d->red[2 * static_cast<size_t>(c) + 1];
    }
    s = warp_sum(s);
    n = warp_sum(n);
    if (lane == 0) d->st[p].fitness = n > 0 ? s / n : DBL_MAX;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt->fit_tile_ctr = 0;
    cnt->nfar = 0;
    cnt->far_ctr = 0;
  }
}

// Target centroids of every pair (the centre of the linear algebra), FP64:
// chunks of 2048 target points give partial (x, y, z, count) sums (threads
// stride the chunk, fixed tree), then one warp per pair adds its chunks in
// order and writes the mean as float into prm.
constexpr int kCentroidChunk = 2048;

__global__ void __launch_bounds__(kIcpThreads) k_centroid_chunks(const float4* const* __restrict__ xyz,
                                                                 const int* __restrict__ npts,
                                                                 const int* __restrict__ cc0, int npairs,
                                                                 double* __restrict__ part) {
  __shared__ double s[4][kIcpWarps];
  for (int c = blockIdx.x; c < cc0[npairs]; c += gridDim.x) {
    const int p = pair_of(cc0, npairs, c);
    const float4* __restrict__ x = xyz[p];
    const int i0 = (c - cc0[p]) * kCentroidChunk, i1 = min(npts[p], i0 + kCentroidChunk);
    double a = 0, b = 0, z = 0, w = 0;
    for (int i = i0 + static_cast<int>(threadIdx.x); i < i1; i += blockDim.x) {
      const float4 v = x[i];
      if (!finite3(v.x, v.y, v.z)) continue;
      a += v.x; b += v.y; z += v.z; w += 1.0;
    }
    a = warp_sum(a); b = warp_sum(b); z = warp_sum(z); w = warp_sum(w);
    if ((threadIdx.x & 31) == 0) {
      s[0][threadIdx.x >> 5] = a; s[1][threadIdx.x >> 5] = b;
      s[2][threadIdx.x >> 5] = z; s[3][threadIdx.x >> 5] = w;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
      double v = 0.0;
      for (int k = 0; k < kIcpWarps; ++k) v += s[threadIdx.x][k];
      part[4 * static_cast<size_t>(c) + threadIdx.x] = v;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kIcpThreads) k_centroid_final(const BatchDesc* __restrict__ d,
                                                                const int* __restrict__ cc0,
                                                                const double* __restrict__ part) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int p = warp; p < d->npairs; p += nwarps) {
    double v[4] = {0, 0, 0, 0};
    for (int c = cc0[p] + lane; c < cc0[p + 1]; c += 32)
      for (int k = 0; k < 4; ++k) v[k] += part[4 * static_cast<size_t>(c) + k];
    for (int k = 0; k < 4; ++k) v[k] = warp_sum(v[k]);
    if (lane < 3) {
      const double m = v[3] > 0 ? v[lane] / v[3] : 0.0;
      d->prm[p].c[lane] = static_cast<float>(m);
    }
  }
}

int icp_grid(lcr_ctx* ctx) { return ctx->sms * ctx->tune.icp_bps; }
int reduce_grid(lcr_ctx* ctx) { return ctx->sms * 2; }

// Persistent per-context block: the descriptor, then the counters.
struct IcpBuffers {
  BatchDesc* desc;
  BatchCounters* cnt;
};

IcpBuffers icp_buffers(lcr_ctx* ctx) {
  static_assert(sizeof(BatchDesc) <= 512 && sizeof(BatchCounters) <= 512, "ICP structs must fit their slots");
  if (!ctx->icp_block) {
    CUDA_TRY(cudaMalloc(&ctx->icp_block, 1024));
    CUDA_TRY(cudaMemsetAsync(ctx->icp_block, 0, 1024, ctx->stream));
    ctx->icp_bytes = 1024;
  }
  char* b = static_cast<char*>(ctx->icp_block);
  return IcpBuffers{reinterpret_cast<BatchDesc*>(b), reinterpret_cast<BatchCounters*>(b + 512)};
}

// Solve blocks of a round: one per pair, up to 1024 (more pairs loop).
int solve_blocks(int npairs) { return npairs <= 1 ? 1 : (npairs <= 64 ? 64 : 1024); }
int solve_slot(int blocks) { return blocks == 1 ? 0 : (blocks == 64 ? 1 : 2); }

// Builds (once per context, method and solve width) the graph
// WHILE(cond) { search; hard; wide; reduce; solve }.  Returns nullptr if
// conditional nodes are unavailable.
cudaGraphExec_t icp_graph(lcr_ctx* ctx, int p2pl, int sblocks, const IcpBuffers& B) {
  // LCR_ICP_GRAPH=0 runs the same kernels from a host loop instead (profilers
  // do not see kernels inside conditional graph bodies).
  const char* env = std::getenv("LCR_ICP_GRAPH");
  if (env && env[0] == '0') return nullptr;
  if (ctx->icp_graph_ok == 0) return nullptr;
  cudaGraphExec_t& slot = ctx->icp_exec[p2pl][solve_slot(sblocks)];
  if (slot) return slot;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
  cudaGraphConditionalHandle h = 0;
  if (ok) ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  // cudaGraphNodeParams has no usable default constructor: zeroed raw storage.
  alignas(cudaGraphNodeParams) unsigned char cp_raw[sizeof(cudaGraphNodeParams)];
  std::memset(cp_raw, 0, sizeof(cp_raw));
  cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cp_raw);
  cudaGraphNode_t wnode = nullptr;
  if (ok) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    ok = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const BatchDesc* a0 = B.desc;
    BatchCounters* a1 = B.cnt;
    void* args2[] = {&a0, &a1};
    void* args3[] = {&a0, &a1, &h};
    struct NodeSpec { void* fn; int grid; void** args; };
    const NodeSpec specs[5] = {
        {p2pl ? reinterpret_cast<void*>(k_icp_search<1>) : reinterpret_cast<void*>(k_icp_search<0>), icp_grid(ctx), args2},
        {reinterpret_cast<void*>(k_icp_hard), icp_grid(ctx), args2},
        {p2pl ? reinterpret_cast<void*>(k_icp_wide<1>) : reinterpret_cast<void*>(k_icp_wide<0>), icp_grid(ctx), args2},
        {reinterpret_cast<void*>(k_icp_reduce), reduce_grid(ctx), args2},
        {p2pl ? reinterpret_cast<void*>(k_icp_solve<1>) : reinterpret_cast<void*>(k_icp_solve<0>), sblocks, args3}};
    cudaGraphNode_t prev = nullptr;
    for (int k = 0; k < 5 && ok; ++k) {
      cudaKernelNodeParams kp;
      std::memset(&kp, 0, sizeof(kp));
      kp.func = specs[k].fn;
      kp.gridDim = dim3(specs[k].grid);
      kp.blockDim = dim3(kIcpThreads);
      kp.kernelParams = specs[k].args;
      cudaGraphNode_t node = nullptr;
      ok = cudaGraphAddKernelNode(&node, body, prev ? &prev : nullptr, prev ? 1 : 0, &kp) == cudaSuccess;
      prev = node;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    ctx->icp_graph_ok = 0;
    return nullptr;
  }
  ctx->icp_graph_ok = 1;
  slot = exec;
  return exec;
}

inline size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }

}  // namespace

float float_cap(double v);

void icp_batch_run(lcr_ctx* ctx, const lcr_cloud* const* src, const lcr_cloud* const* tgt, int npairs,
                   const lcr_icp_params* p, const float* guesses, lcr_icp_result* res) {
  if (p->max_iterations <= 0) LCR_THROW(LCR_ERR_INVALID_ARG, "max_iterations needs to be greater than zero");
  if (!(p->max_correspondence_distance >= 0)) LCR_THROW(LCR_ERR_INVALID_ARG, "negative correspondence distance");
  if (npairs <= 0) return;
  for (int i = 0; i < npairs; ++i)
    if (!src[i] || !tgt[i]) LCR_THROW(LCR_ERR_INVALID_ARG, "null cloud in pair %d", i);
  for (int i = 0; i < npairs; ++i)
    if (src[i]->n == 0 || tgt[i]->n == 0) LCR_THROW(LCR_ERR_EMPTY, "ICP needs non-empty source and target clouds (pair %d)", i);
  const int p2pl = p->method == LCR_ICP_POINT_TO_PLANE ? 1 : 0;
  const IcpBuffers B = icp_buffers(ctx);
  const int sblocks = solve_blocks(npairs);
  cudaGraphExec_t exec = icp_graph(ctx, p2pl, sblocks, B);

  // host staging: pair parameters, states, prefixes, centroid inputs
  std::vector<IcpParams> hp(npairs);
  std::vector<IcpState> hs(npairs);
  std::vector<int> tile0(npairs + 1), chunk0(npairs + 1), npts(npairs), cc0(npairs + 1, 0);
  std::vector<const float4*> txyz(npairs);
  const float cap = float_cap(p->max_correspondence_distance * p->max_correspondence_distance);
  int tiles = 0, chunks = 0;
  for (int i = 0; i < npairs; ++i) {
    const Index& si = cloud_index(ctx, src[i]);
    const Index& ti = cloud_index(ctx, tgt[i]);
    IcpParams& q = hp[i];
    std::memset(&q, 0, sizeof(q));
    q.tgt = ti.v;
    q.src_pts = si.v.pts;
    q.tgt_nrm = tgt[i]->nrm;
    q.tgt_xyz = tgt[i]->xyz;
    q.src_ntiles = si.v.nleaf;
    q.tile0 = tiles;
    q.chunk0 = chunks;
    q.cap = cap;
    q.min_corr = 3;
    q.max_iter = p->max_iterations;
    q.teps = p->transformation_epsilon;
    q.feps = p->euclidean_fitness_epsilon;
    q.stop_iter = p->stop_iteration;
    q.stop_mse = p->stop_rms * p->stop_rms;
    if (tgt[i]->graph) {
      q.tgt_rows = tgt[i]->graph->rows;
      q.tgt_k = tgt[i]->graph->k;
    }
    tile0[i] = tiles;
    chunk0[i] = chunks;
    tiles += si.v.nleaf;
    chunks += (si.v.nleaf + kChunkTiles - 1) / kChunkTiles;
    IcpState& s = hs[i];
    std::memset(&s, 0, sizeof(s));
    const double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (int k = 0; k < 16; ++k) s.T[k] = guesses ? static_cast<double>(guesses[16 * i + k]) : I[k];
    for (int k = 0; k < 12; ++k) s.Tf.m[k] = static_cast<float>(s.T[k]);
    s.prev_mse = DBL_MAX;
    txyz[i] = tgt[i]->xyz;
    npts[i] = static_cast<int>(tgt[i]->n);
    cc0[i + 1] = cc0[i] + (npts[i] + kCentroidChunk - 1) / kCentroidChunk;
  }
  tile0[npairs] = tiles;
  chunk0[npairs] = chunks;
  const int cchunks = cc0[npairs];
  const size_t slots = static_cast<size_t>(tiles) * 32;

  // one device block for the call: pair arrays, then the scratch
  const size_t b_prm = align256(sizeof(IcpParams) * npairs), b_st = align256(sizeof(IcpState) * npairs),
               b_pre = align256(sizeof(int) * (npairs + 1)), b_xyz = align256(sizeof(float4*) * npairs),
               b_npts = align256(sizeof(int) * npairs), b_part = align256(slots * 4), b_hq = align256(slots * 4),
               b_htp = align256(slots * 16), b_hti = align256(slots * 4), b_wide = align256(sizeof(uint32_t) * tiles),
               b_red = align256(sizeof(double) * 32 * chunks), b_fd = align256(slots * 4),
               b_far = align256(slots * 16), b_cpart = align256(sizeof(double) * 4 * cchunks),
               b_prev = align256(slots * 4);
  const size_t hdr = b_prm + b_st + 3 * b_pre + b_xyz + b_npts;
  char* blk = static_cast<char*>(
      dev_alloc(ctx, hdr + b_part + b_hq + b_htp + b_hti + b_wide + b_red + b_fd + b_far + b_cpart + b_prev));
  char* cur = blk;
  BatchDesc hd;
  std::memset(&hd, 0, sizeof(hd));
  hd.npairs = npairs;
  hd.total_tiles = tiles;
  hd.total_chunks = chunks;
  hd.use_graph = exec ? 1 : 0;
  hd.prm = reinterpret_cast<IcpParams*>(cur); cur += b_prm;
  hd.st = reinterpret_cast<IcpState*>(cur); cur += b_st;
  int* d_tile0 = reinterpret_cast<int*>(cur); cur += b_pre;
  int* d_chunk0 = reinterpret_cast<int*>(cur); cur += b_pre;
  const float4** d_xyz = reinterpret_cast<const float4**>(cur); cur += b_xyz;
  int* d_npts = reinterpret_cast<int*>(cur); cur += b_npts;
  int* d_cc0 = reinterpret_cast<int*>(cur); cur += b_pre;
  hd.tile0 = d_tile0;
  hd.chunk0 = d_chunk0;
  hd.tile_part = reinterpret_cast<float*>(cur); cur += b_part;
  hd.hard_q = reinterpret_cast<uint32_t*>(cur); cur += b_hq;
  hd.hard_tp = reinterpret_cast<float4*>(cur); cur += b_htp;
  hd.hard_ti = reinterpret_cast<uint32_t*>(cur); cur += b_hti;
  hd.wide_tiles = reinterpret_cast<uint32_t*>(cur); cur += b_wide;
  hd.red = reinterpret_cast<double*>(cur); cur += b_red;
  hd.fd = reinterpret_cast<float*>(cur); cur += b_fd;
  hd.far = reinterpret_cast<float4*>(cur); cur += b_far;
  double* d_cpart = reinterpret_cast<double*>(cur); cur += b_cpart;
  hd.prev_ti = reinterpret_cast<uint32_t*>(cur);
  CUDA_TRY(cudaMemsetAsync(hd.prev_ti, 0xff, slots * 4, ctx->stream));

  // stage everything in one pinned buffer and copy it in one go
  const size_t stage_bytes = hdr + 1024 + 256;
  char* stage = static_cast<char*>(pinned(ctx, stage_bytes));
  std::memset(stage, 0, stage_bytes);
  std::memcpy(stage, hp.data(), sizeof(IcpParams) * npairs);
  std::memcpy(stage + b_prm, hs.data(), sizeof(IcpState) * npairs);
  std::memcpy(stage + b_prm + b_st, tile0.data(), sizeof(int) * (npairs + 1));
  std::memcpy(stage + b_prm + b_st + b_pre, chunk0.data(), sizeof(int) * (npairs + 1));
  std::memcpy(stage + b_prm + b_st + 2 * b_pre, txyz.data(), sizeof(float4*) * npairs);
  std::memcpy(stage + b_prm + b_st + 2 * b_pre + b_xyz, npts.data(), sizeof(int) * npairs);
  std::memcpy(stage + b_prm + b_st + 2 * b_pre + b_xyz + b_npts, cc0.data(), sizeof(int) * (npairs + 1));
  BatchCounters hc;
  std::memset(&hc, 0, sizeof(hc));
  hc.max_rounds = p->max_iterations + 1;
  std::memcpy(stage + hdr, &hd, sizeof(hd));
  std::memcpy(stage + hdr + 512, &hc, sizeof(hc));
  CUDA_TRY(cudaMemcpyAsync(blk, stage, hdr, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(B.desc, stage + hdr, 1024, cudaMemcpyHostToDevice, ctx->stream));
  const int pair_blocks = std::min((npairs + kIcpWarps - 1) / kIcpWarps, 128);  // one warp per pair
  LCR_LAUNCH(ctx, k_centroid_chunks, std::min(cchunks, icp_grid(ctx)), kIcpThreads, 0, d_xyz, d_npts, d_cc0, npairs,
             d_cpart);
  LCR_LAUNCH(ctx, k_centroid_final, pair_blocks, kIcpThreads, 0, B.desc, d_cc0, d_cpart);

  if (exec) {
    CUDA_TRY(cudaGraphLaunch(exec, ctx->stream));
  } else {
    cudaGraphConditionalHandle none = 0;
    const int grid = icp_grid(ctx);
    unsigned* hlive = reinterpret_cast<unsigned*>(stage + hdr + 1024);
    for (int it = 0; it < p->max_iterations + 1; ++it) {
      {
        KernelTimer kt(ctx, LCR_KT_ICP_SEARCH);
        if (p2pl) LCR_LAUNCH(ctx, k_icp_search<1>, grid, kIcpThreads, 0, B.desc, B.cnt);
        else LCR_LAUNCH(ctx, k_icp_search<0>, grid, kIcpThreads, 0, B.desc, B.cnt);
      }
      LCR_LAUNCH(ctx, k_icp_hard, grid, kIcpThreads, 0, B.desc, B.cnt);
      if (p2pl) LCR_LAUNCH(ctx, k_icp_wide<1>, grid, kIcpThreads, 0, B.desc, B.cnt);
      else LCR_LAUNCH(ctx, k_icp_wide<0>, grid, kIcpThreads, 0, B.desc, B.cnt);
      LCR_LAUNCH(ctx, k_icp_reduce, reduce_grid(ctx), kIcpThreads, 0, B.desc, B.cnt);
      if (p2pl) LCR_LAUNCH(ctx, k_icp_solve<1>, sblocks, kIcpThreads, 0, B.desc, B.cnt, none);
      else LCR_LAUNCH(ctx, k_icp_solve<0>, sblocks, kIcpThreads, 0, B.desc, B.cnt, none);
      if ((it & 7) == 7 || it == p->max_iterations) {
        CUDA_TRY(cudaMemcpyAsync(hlive, &B.cnt->live, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        if (*hlive == 0) break;
      }
    }
  }
  if (p->compute_fitness) {
    const int grid = icp_grid(ctx);
    LCR_LAUNCH(ctx, k_fitness, grid, kIcpThreads, 0, B.desc, B.cnt);
    LCR_LAUNCH(ctx, k_fitness_far, grid, kIcpThreads, 0, B.desc, B.cnt);
    LCR_LAUNCH(ctx, k_fitness_chunks, reduce_grid(ctx), kIcpThreads, 0, B.desc);
    LCR_LAUNCH(ctx, k_fitness_reduce, pair_blocks, kIcpThreads, 0, B.desc, B.cnt);
  }
  IcpState* out = reinterpret_cast<IcpState*>(stage);  // after the staged copy in stream order
  unsigned* hrounds = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(out) + b_st);
  CUDA_TRY(cudaMemcpyAsync(out, hd.st, sizeof(IcpState) * npairs, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(hrounds, &B.cnt->rounds, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  dev_free(ctx, blk);
  sync(ctx);
  if (exec) ctx->launches += 5 * static_cast<uint64_t>(*hrounds);  // five kernels per body run
  for (int i = 0; i < npairs; ++i) {
    const IcpState& s = out[i];
    lcr_icp_result& r = res[i];
    std::memset(&r, 0, sizeof(r));
    for (int k = 0; k < 16; ++k) {
      r.transform64[k] = s.T[k];
      r.transform[k] = static_cast<float>(s.T[k]);
    }
    r.converged = s.converged;
    r.iterations = s.iter;
    r.state = s.state;
    r.n_correspondences = s.ncorr;
    r.fitness = p->compute_fitness ? s.fitness : 0.0;
    r.mse = s.mse;
  }
}

void icp_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const lcr_icp_params* p, const float* guess,
             lcr_icp_result* res) {
  icp_batch_run(ctx, &src, &tgt, 1, p, guess, res);
}

void icp_graphs_reset(lcr_ctx* ctx) {
  for (auto& per_method : ctx->icp_exec)
    for (cudaGraphExec_t& e : per_method)
      if (e) {
        cudaGraphExecDestroy(e);
        e = nullptr;
      }
}
