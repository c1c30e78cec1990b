// pcl::IterativeClosestPoint on the GPU (pcl_tools/fine_registration.cpp:105-126).
//
// One ICP iteration is five launches, captured once per context as the body of
// a CUDA-graph WHILE node (LCR_ICP_GRAPH=0 runs them from a host loop):
//  1. k_icp_search  warps take tiles of 32 Hilbert-sorted source points,
//                   transform them by the current FP32 transform, find each
//                   point's exact nearest target within the correspondence
//                   distance (one shared warp-tile traversal), form the
//                   per-correspondence terms in FP32 and reduce them across the
//                   warp with a transposing reduce-scatter (lane l ends with
//                   term l) into a per-tile row.  Tiles wider than four search
//                   radii are deferred.
//  2. k_icp_hard    one warp per point of a deferred tile (per-query pruning).
//  3. k_icp_wide    the term rows of the deferred tiles.
//  4. k_icp_reduce  fixed-order FP64 sums of the tile rows.
//  5. k_icp_solve   one block: FP64 solve (3x3 SVD for point-to-point, 6x6
//                   LDL^T for point-to-plane), compose, re-orthonormalise, PCL's
//                   DefaultConvergenceCriteria, and the WHILE condition.
// Every sum runs in a fixed order, so the result does not depend on scheduling.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "search.cuh"

namespace {

constexpr int kIcpThreads = 256;
constexpr int kIcpWarps = kIcpThreads / 32;
constexpr int kIcpReduceBlocks = 128;

struct IcpParams {
  IndexView tgt;
  const float4* src_pts;  // Morton-sorted source (the source index's points)
  int src_ntiles;
  const float4* tgt_nrm;  // target normals by original index
  float cap;              // FP32 form of max_correspondence_distance^2
  float c[3];             // fixed centre of the linear algebra: target centroid (float)
  int min_corr;
  int max_iter;
  double teps, feps;
  int use_graph;
  float* fd;              // fitness: squared NN distance per sorted source slot
  float4* far;            // fitness: queries with no target point inside the cap
  float* tile_part;       // per-tile FP32 term sums [ntiles][32]
  uint32_t* hard_q;       // deferred query slots (points of wide tiles)
  float4* hard_tp;        // per-slot result of a deferred query: target xyz, distance
  uint32_t* hard_ti;      // per-slot target index (0xffffffff: none within the cap)
  uint32_t* wide_tiles;   // tiles whose terms wait for the deferred queries
};

struct IcpState {
  double T[16];
  Xf Tf;
  double prev_mse, mse, fitness;
  int iter, done, converged, state, ncorr, launches;
  unsigned int tile_ctr, blocks_done;
  unsigned int fit_tile_ctr, fit_blocks_done, nfar, far_ctr;
  unsigned int nhard, hard_ctr, nwide, wide_ctr;
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
__device__ bool ldlt6(const double M[36], const double b[6], double x[6]) {
  double L[36], D[6];
  double dmax = 0;
  for (int i = 0; i < 6; ++i) dmax = fmax(dmax, fabs(M[7 * i]));
  if (!(dmax > 0)) return false;
  for (int i = 0; i < 36; ++i) L[i] = 0;
  for (int j = 0; j < 6; ++j) {
    double d = M[6 * j + j];
    for (int k = 0; k < j; ++k) d -= L[6 * j + k] * L[6 * j + k] * D[k];
    if (!(d > 1e-12 * dmax)) return false;
    D[j] = d;
    L[6 * j + j] = 1.0;
    for (int i = j + 1; i < 6; ++i) {
      double v = M[6 * i + j];
      for (int k = 0; k < j; ++k) v -= L[6 * i + k] * L[6 * j + k] * D[k];
      L[6 * i + j] = v / d;
    }
  }
  double y[6];
  for (int i = 0; i < 6; ++i) {
    double v = b[i];
    for (int k = 0; k < i; ++k) v -= L[6 * i + k] * y[k];
    y[i] = v;
  }
  for (int i = 0; i < 6; ++i) y[i] /= D[i];
  for (int i = 5; i >= 0; --i) {
    double v = y[i];
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
__device__ bool solve_plane(const double* S, const double c[3], double dT[16]) {
  double M[36], b[6], x[6];
  int k = 0;
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j) {
      M[6 * i + j] = S[k];
      M[6 * j + i] = S[k];
      ++k;
    }
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

__device__ void orthonormalize(double T[16]) {
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
__device__ void icp_update(const double* S, const IcpParams* prm, IcpState* st) {
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
  double T[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += dT[4 * i + k] * st->T[4 * k + j];
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

__device__ __forceinline__ bool icp_done(const IcpState* st) {
  return *reinterpret_cast<const volatile int*>(&st->done) != 0;
}

// Pass 1 of an iteration.  Warps take tiles of 32 Morton-sorted source points
// dynamically; a compact tile shares one capped 1-NN traversal and stores its
// 32 FP32 term sums (lane l = term l) in tile_part[tile].  A tile wider than
// four search radii (its queries straddle distant surfaces) is deferred: its
// points go to the hard-query list and the tile to the wide list.
template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_search(const IcpParams* __restrict__ prm, IcpState* st) {
  __shared__ IndexView s_tgt;
  __shared__ Xf s_T;
  __shared__ WarpScratch wss[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (icp_done(st)) return;
  if (threadIdx.x == 0) {
    s_tgt = prm->tgt;
    s_T = st->Tf;
  }
  __syncthreads();
  const float4* __restrict__ src = prm->src_pts;
  const int ntiles = prm->src_ntiles;
  const float cap = prm->cap;
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = static_cast<int>(atomicAdd(&st->tile_ctr, 1u));
    tile = __shfl_sync(LCR_FULL, tile, 0);
    if (tile >= ntiles) break;
    const int slot = tile * 32 + lane;
    const float4 p = src[slot];
    const bool pv = finite3(p.x, p.y, p.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    if (pv) q = xf_apply(s_T, p.x, p.y, p.z);
    float4 tlo, thi;
    if (!tile_box(q.x, q.y, q.z, pv, tlo, thi)) {
      prm->tile_part[slot] = 0.f;
      continue;
    }
    const float dx = thi.x - tlo.x, dy = thi.y - tlo.y, dz = thi.z - tlo.z;
    if (dx * dx + dy * dy + dz * dz > 16.f * cap) {
      const unsigned valid = __ballot_sync(LCR_FULL, pv);
      unsigned base = 0;
      if (lane == 0) {
        base = atomicAdd(&st->nhard, static_cast<unsigned>(__popc(valid)));
        prm->wide_tiles[atomicAdd(&st->nwide, 1u)] = static_cast<uint32_t>(tile);
      }
      base = __shfl_sync(LCR_FULL, base, 0);
      if (pv) prm->hard_q[base + __popc(valid & ((1u << lane) - 1u))] = static_cast<uint32_t>(slot);
      continue;
    }
    NN1 v;
    v.init(q.x, q.y, q.z, pv, cap, wss[wib]);
    tile_traverse(s_tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), wss[wib]);
    float t[32];
    corr_terms<P2PL>(t, pv && v.found(), q, v.bp, key_dist(v.best), key_idx(v.best), prm);
    prm->tile_part[slot] = reduce_scatter32(t, lane);
  }
}

// Pass 2: the deferred queries, one per warp (exact per-query pruning), spread
// over the whole grid; results land in per-point slots.
__global__ void __launch_bounds__(kIcpThreads) k_icp_hard(const IcpParams* __restrict__ prm, IcpState* st) {
  __shared__ IndexView s_tgt;
  __shared__ Xf s_T;
  __shared__ WarpScratch wss[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (icp_done(st)) return;
  if (threadIdx.x == 0) {
    s_tgt = prm->tgt;
    s_T = st->Tf;
  }
  __syncthreads();
  const unsigned nhard = *reinterpret_cast<volatile unsigned*>(&st->nhard);
  for (;;) {
    unsigned i = 0;
    if (lane == 0) i = atomicAdd(&st->hard_ctr, 1u);
    i = __shfl_sync(LCR_FULL, i, 0);
    if (i >= nhard) break;
    const uint32_t slot = prm->hard_q[i];
    const float4 p = prm->src_pts[slot];
    const float3 q = xf_apply(s_T, p.x, p.y, p.z);
    unsigned long long best;
    float4 bp;
    warp_query_nn(s_tgt, q.x, q.y, q.z, prm->cap, wss[wib], best, bp);
    if (lane == 0) {
      prm->hard_tp[slot] = make_float4(bp.x, bp.y, bp.z, key_dist(best));
      prm->hard_ti[slot] = key_idx(best);
    }
  }
}

// Pass 3: term sums of the wide tiles from the per-point results.
template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_wide(const IcpParams* __restrict__ prm, IcpState* st) {
  __shared__ Xf s_T;
  const int lane = threadIdx.x & 31;
  if (icp_done(st)) return;
  if (threadIdx.x == 0) s_T = st->Tf;
  __syncthreads();
  const unsigned nwide = *reinterpret_cast<volatile unsigned*>(&st->nwide);
  for (;;) {
    unsigned i = 0;
    if (lane == 0) i = atomicAdd(&st->wide_ctr, 1u);
    i = __shfl_sync(LCR_FULL, i, 0);
    if (i >= nwide) break;
    const int slot = static_cast<int>(prm->wide_tiles[i]) * 32 + lane;
    const float4 p = prm->src_pts[slot];
    const bool pv = finite3(p.x, p.y, p.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    float4 tp = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t ti = 0xffffffffu;
    if (pv) {
      q = xf_apply(s_T, p.x, p.y, p.z);
      tp = prm->hard_tp[slot];
      ti = prm->hard_ti[slot];
    }
    float t[32];
    corr_terms<P2PL>(t, pv && ti != 0xffffffffu, q, tp, tp.w, ti, prm);
    prm->tile_part[slot] = reduce_scatter32(t, lane);
  }
}

// Pass 4: fixed-order FP64 reduction of the per-tile sums: block b owns a
// contiguous range of tiles, 8 sub-slices x 32 terms per block.
__global__ void __launch_bounds__(256) k_icp_reduce(const IcpParams* __restrict__ prm, const IcpState* st,
                                                   double* __restrict__ red) {
  __shared__ double s[8][32];
  if (icp_done(st)) return;
  const int ntiles = prm->src_ntiles;
  const int chunk = (ntiles + gridDim.x - 1) / gridDim.x;
  const int t0 = blockIdx.x * chunk, t1 = min(ntiles, t0 + chunk);
  const int term = threadIdx.x & 31, sub = threadIdx.x >> 5;
  double acc = 0.0;
  for (int t = t0 + sub; t < t1; t += 8) acc += static_cast<double>(prm->tile_part[t * 32 + term]);
  s[sub][term] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) v += s[k][threadIdx.x];
    red[blockIdx.x * 32 + threadIdx.x] = v;
  }
}

// Pass 5, one block: sum of the block partials in order, FP64 solve, compose,
// convergence test, counters reset, and the loop condition for the graph.
template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_solve(const IcpParams* __restrict__ prm, IcpState* st,
                                                           const double* __restrict__ red, int nred,
                                                           cudaGraphConditionalHandle h) {
  __shared__ double s_acc[kIcpWarps][32];
  if (icp_done(st)) {
    if (threadIdx.x == 0 && prm->use_graph) cudaGraphSetConditional(h, 0u);
    return;
  }
  const int term = threadIdx.x & 31, slice = threadIdx.x >> 5;
  double s = 0.0;
  for (int b = slice; b < nred; b += kIcpWarps) s += red[static_cast<size_t>(b) * 32 + term];
  s_acc[slice][term] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double S[32];
    for (int t = 0; t < 32; ++t) {
      double v = 0.0;
      for (int w = 0; w < kIcpWarps; ++w) v += s_acc[w][t];
      S[t] = v;
    }
    icp_update<P2PL>(S, prm, st);
    st->launches += 1;
    if (st->launches > prm->max_iter + 1) st->done = 1;  // hard bound on the device loop
    st->tile_ctr = 0;
    st->nhard = 0;
    st->hard_ctr = 0;
    st->nwide = 0;
    st->wide_ctr = 0;
    if (prm->use_graph) cudaGraphSetConditional(h, st->done ? 0u : 1u);
  }
}

// getFitnessScore(): mean squared distance from every transformed source point
// to its exact (uncapped) nearest target point.  Phase 1 searches the tiles with
// the correspondence cap (a far lane would otherwise widen its whole tile's
// search); lanes with no target point inside the cap are queued and phase 2
// finds their nearest point with one warp per query (per-query pruning, the 32
// lanes scan a leaf together).  Distances land in fd[] by sorted source
// position and are summed in a fixed order.  The points of a tile wider than
// four search radii go straight to phase 2.
__global__ void __launch_bounds__(kIcpThreads) k_fitness(const IcpParams* __restrict__ prm, IcpState* st) {
  __shared__ IndexView s_tgt;
  __shared__ Xf s_T;
  __shared__ WarpScratch wss[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_tgt = prm->tgt;
    s_T = st->Tf;
  }
  __syncthreads();
  const float4* __restrict__ src = prm->src_pts;
  const int ntiles = prm->src_ntiles;
  float* __restrict__ fd = prm->fd;
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = static_cast<int>(atomicAdd(&st->fit_tile_ctr, 1u));
    tile = __shfl_sync(LCR_FULL, tile, 0);
    if (tile >= ntiles) break;
    const int pos = tile * 32 + lane;
    const float4 p = src[pos];
    const bool pv = finite3(p.x, p.y, p.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    if (pv) q = xf_apply(s_T, p.x, p.y, p.z);
    float4 tlo, thi;
    if (!tile_box(q.x, q.y, q.z, pv, tlo, thi)) {
      fd[pos] = -1.f;
      continue;
    }
    const float dx = thi.x - tlo.x, dy = thi.y - tlo.y, dz = thi.z - tlo.z;
    if (dx * dx + dy * dy + dz * dz > 16.f * prm->cap) {
      // wide tile: every point goes to the per-query phase (same exact result)
      if (pv) prm->far[atomicAdd(&st->nfar, 1u)] = make_float4(q.x, q.y, q.z, __int_as_float(pos));
      else fd[pos] = -1.f;
      continue;
    }
    NN1 v;
    v.init(q.x, q.y, q.z, pv, prm->cap, wss[wib]);
    tile_traverse(s_tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), wss[wib]);
    if (!pv) {
      fd[pos] = -1.f;  // not a point
    } else if (v.found()) {
      fd[pos] = key_dist(v.best);
    } else {
      const unsigned slot = atomicAdd(&st->nfar, 1u);
      prm->far[slot] = make_float4(q.x, q.y, q.z, __int_as_float(pos));
    }
  }
}

__global__ void __launch_bounds__(kIcpThreads) k_fitness_far(const IcpParams* __restrict__ prm, IcpState* st) {
  __shared__ IndexView s_tgt;
  __shared__ WarpScratch wss[kIcpWarps];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tgt = prm->tgt;
  __syncthreads();
  const unsigned nfar = *reinterpret_cast<volatile unsigned*>(&st->nfar);
  for (;;) {
    unsigned i = 0;
    if (lane == 0) i = atomicAdd(&st->far_ctr, 1u);
    i = __shfl_sync(LCR_FULL, i, 0);
    if (i >= nfar) break;
    const float4 q = prm->far[i];
    unsigned long long best;
    float4 bp;
    warp_query_nn(s_tgt, q.x, q.y, q.z, LCR_INF, wss[wib], best, bp);
    if (lane == 0) prm->fd[__float_as_int(q.w)] = key_dist(best);
  }
}

// Fixed-order FP64 sum of fd[] (negative entries are not points): contiguous
// chunks per block, fixed tree inside the block, blocks added in order by the
// last block.
__global__ void __launch_bounds__(256) k_fitness_reduce(const IcpParams* __restrict__ prm, IcpState* st,
                                                        double* __restrict__ part) {
  __shared__ double s_s[8], s_c[8];
  __shared__ int s_flag;
  const int n = prm->src_ntiles * 32;
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  double s = 0.0, c = 0.0;
  for (int i = b0 + static_cast<int>(threadIdx.x); i < b1; i += blockDim.x) {
    const float d = prm->fd[i];
    if (d >= 0.f) {
      s += d;
      c += 1.0;
    }
  }
  s = warp_sum(s);
  c = warp_sum(c);
  if ((threadIdx.x & 31) == 0) {
    s_s[threadIdx.x >> 5] = s;
    s_c[threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ts = 0.0, tc = 0.0;
    for (int w = 0; w < 8; ++w) {
      ts += s_s[w];
      tc += s_c[w];
    }
    part[2 * blockIdx.x] = ts;
    part[2 * blockIdx.x + 1] = tc;
    __threadfence();
    s_flag = (atomicAdd(&st->fit_blocks_done, 1u) == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (!s_flag || threadIdx.x != 0) return;
  __threadfence();
  double ts = 0.0, tc = 0.0;
  for (int b = 0; b < static_cast<int>(gridDim.x); ++b) {
    ts += __ldcg(&part[2 * b]);
    tc += __ldcg(&part[2 * b + 1]);
  }
  st->fitness = tc > 0 ? ts / tc : DBL_MAX;
  st->fit_tile_ctr = 0;
  st->fit_blocks_done = 0;
  st->nfar = 0;
  st->far_ctr = 0;
}

struct IcpBuffers {
  IcpParams* prm;
  IcpState* st;
  double* part;
};

IcpBuffers icp_buffers(lcr_ctx* ctx, int grid) {
  const size_t need = 1024 + 1024 + static_cast<size_t>(grid) * 32 * sizeof(double);
  if (ctx->icp_bytes < need) {
    if (ctx->icp_block) {
      sync(ctx);
      CUDA_TRY(cudaFree(ctx->icp_block));
      for (int m = 0; m < 2; ++m)
        if (ctx->icp_exec[m]) {
          cudaGraphExecDestroy(ctx->icp_exec[m]);
          ctx->icp_exec[m] = nullptr;
        }
    }
    CUDA_TRY(cudaMalloc(&ctx->icp_block, need));
    CUDA_TRY(cudaMemsetAsync(ctx->icp_block, 0, need, ctx->stream));
    ctx->icp_bytes = need;
  }
  char* b = static_cast<char*>(ctx->icp_block);
  static_assert(sizeof(IcpParams) <= 1024 && sizeof(IcpState) <= 1024, "ICP structs must fit their slots");
  return IcpBuffers{reinterpret_cast<IcpParams*>(b), reinterpret_cast<IcpState*>(b + 1024),
                    reinterpret_cast<double*>(b + 2048)};
}

int icp_grid(lcr_ctx* ctx) { return ctx->sms * 4; }

// Builds (once per context and method) the graph WHILE(cond) { iteration }.
// Returns nullptr if conditional nodes are unavailable.
cudaGraphExec_t icp_graph(lcr_ctx* ctx, int p2pl, const IcpBuffers& B) {
  // LCR_ICP_GRAPH=0 runs the same iteration kernels from a host loop instead
  // (profilers do not see kernels inside conditional graph bodies).
  const char* env = std::getenv("LCR_ICP_GRAPH");
  if (env && env[0] == '0') return nullptr;
  if (ctx->icp_graph_ok == 0) return nullptr;
  if (ctx->icp_exec[p2pl]) return ctx->icp_exec[p2pl];
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
    // body: search, deferred queries, wide-tile terms, fixed-order reduction,
    // then the one-block FP64 solve that sets the loop condition.
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const IcpParams* a0 = B.prm;
    IcpState* a1 = B.st;
    double* a2 = B.part;
    int a3 = kIcpReduceBlocks;
    void* args2[] = {&a0, &a1};
    void* args_red[] = {&a0, &a1, &a2};
    void* args_solve[] = {&a0, &a1, &a2, &a3, &h};
    struct NodeSpec { void* fn; int grid; void** args; };
    const NodeSpec specs[5] = {
        {p2pl ? reinterpret_cast<void*>(k_icp_search<1>) : reinterpret_cast<void*>(k_icp_search<0>), icp_grid(ctx), args2},
        {reinterpret_cast<void*>(k_icp_hard), icp_grid(ctx), args2},
        {p2pl ? reinterpret_cast<void*>(k_icp_wide<1>) : reinterpret_cast<void*>(k_icp_wide<0>), icp_grid(ctx), args2},
        {reinterpret_cast<void*>(k_icp_reduce), kIcpReduceBlocks, args_red},
        {p2pl ? reinterpret_cast<void*>(k_icp_solve<1>) : reinterpret_cast<void*>(k_icp_solve<0>), 1, args_solve}};
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
  ctx->icp_exec[p2pl] = exec;
  return exec;
}

}  // namespace

float float_cap(double v);

void icp_run(lcr_ctx* ctx, const lcr_cloud* src, const lcr_cloud* tgt, const lcr_icp_params* p, const float* guess,
             lcr_icp_result* res) {
  if (p->max_iterations <= 0) LCR_THROW(LCR_ERR_INVALID_ARG, "max_iterations needs to be greater than zero");
  if (!(p->max_correspondence_distance >= 0)) LCR_THROW(LCR_ERR_INVALID_ARG, "negative correspondence distance");
  if (src->n == 0 || tgt->n == 0) LCR_THROW(LCR_ERR_EMPTY, "ICP needs non-empty source and target clouds");
  const int p2pl = p->method == LCR_ICP_POINT_TO_PLANE ? 1 : 0;
  const Index& si = cloud_index(ctx, src);
  const Index& ti = cloud_index(ctx, tgt);
  const int grid = icp_grid(ctx);
  IcpBuffers B = icp_buffers(ctx, grid);

  cudaGraphExec_t exec = icp_graph(ctx, p2pl, B);
  char* stage = static_cast<char*>(pinned(ctx, 2048));
  IcpParams* hp = reinterpret_cast<IcpParams*>(stage);
  IcpState* hs = reinterpret_cast<IcpState*>(stage + 1024);
  std::memset(stage, 0, 2048);
  hp->tgt = ti.v;
  hp->src_pts = si.v.pts;
  hp->src_ntiles = si.v.nleaf;
  hp->tgt_nrm = tgt->nrm;
  hp->cap = float_cap(p->max_correspondence_distance * p->max_correspondence_distance);
  hp->min_corr = 3;
  hp->max_iter = p->max_iterations;
  hp->teps = p->transformation_epsilon;
  hp->feps = p->euclidean_fitness_epsilon;
  hp->use_graph = exec ? 1 : 0;
  const size_t nslots = static_cast<size_t>(si.v.nleaf) * 32;
  // per-call scratch: fitness slots + far list, tile sums, deferred queries
  const size_t b_fd = nslots * 4, b_far = nslots * 16, b_part = nslots * 4, b_hq = nslots * 4, b_htp = nslots * 16,
               b_hti = nslots * 4, b_wide = static_cast<size_t>(si.v.nleaf) * 4;
  char* callbuf = static_cast<char*>(dev_alloc(ctx, b_fd + b_far + b_part + b_hq + b_htp + b_hti + b_wide + 256));
  char* cur = callbuf;
  hp->far = reinterpret_cast<float4*>(cur); cur += b_far;
  hp->hard_tp = reinterpret_cast<float4*>(cur); cur += b_htp;
  hp->fd = reinterpret_cast<float*>(cur); cur += b_fd;
  hp->tile_part = reinterpret_cast<float*>(cur); cur += b_part;
  hp->hard_q = reinterpret_cast<uint32_t*>(cur); cur += b_hq;
  hp->hard_ti = reinterpret_cast<uint32_t*>(cur); cur += b_hti;
  hp->wide_tiles = reinterpret_cast<uint32_t*>(cur);
  const double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  for (int i = 0; i < 16; ++i) hs->T[i] = guess ? static_cast<double>(guess[i]) : I[i];
  for (int i = 0; i < 12; ++i) hs->Tf.m[i] = static_cast<float>(hs->T[i]);
  hs->prev_mse = DBL_MAX;
  CUDA_TRY(cudaMemcpyAsync(B.prm, stage, 2048, cudaMemcpyHostToDevice, ctx->stream));
  // centre of the linear algebra: the target centroid (FP64 sums, cast to float)
  double* c4 = static_cast<double*>(dev_alloc(ctx, 4 * sizeof(double)));
  centroid_device(ctx, tgt, c4, &B.prm->c[0]);
  dev_free(ctx, c4);

  if (exec) {
    CUDA_TRY(cudaGraphLaunch(exec, ctx->stream));
  } else {
    cudaGraphConditionalHandle none = 0;
    for (int it = 0; it < p->max_iterations; ++it) {
      if (p2pl) LCR_LAUNCH(ctx, k_icp_search<1>, grid, kIcpThreads, 0, B.prm, B.st);
      else LCR_LAUNCH(ctx, k_icp_search<0>, grid, kIcpThreads, 0, B.prm, B.st);
      LCR_LAUNCH(ctx, k_icp_hard, grid, kIcpThreads, 0, B.prm, B.st);
      if (p2pl) LCR_LAUNCH(ctx, k_icp_wide<1>, grid, kIcpThreads, 0, B.prm, B.st);
      else LCR_LAUNCH(ctx, k_icp_wide<0>, grid, kIcpThreads, 0, B.prm, B.st);
      LCR_LAUNCH(ctx, k_icp_reduce, kIcpReduceBlocks, 256, 0, B.prm, B.st, B.part);
      if (p2pl) LCR_LAUNCH(ctx, k_icp_solve<1>, 1, kIcpThreads, 0, B.prm, B.st, B.part, kIcpReduceBlocks, none);
      else LCR_LAUNCH(ctx, k_icp_solve<0>, 1, kIcpThreads, 0, B.prm, B.st, B.part, kIcpReduceBlocks, none);
      if ((it & 7) == 7) {
        int* hd = static_cast<int*>(pinned(ctx, 2048)) + 384;
        CUDA_TRY(cudaMemcpyAsync(hd, &B.st->done, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        if (*hd) break;
      }
    }
  }
  if (p->compute_fitness) {
    LCR_LAUNCH(ctx, k_fitness, grid, kIcpThreads, 0, B.prm, B.st);
    LCR_LAUNCH(ctx, k_fitness_far, grid, kIcpThreads, 0, B.prm, B.st);
    LCR_LAUNCH(ctx, k_fitness_reduce, std::min(grid, 256), 256, 0, B.prm, B.st, B.part);
  }
  CUDA_TRY(cudaMemcpyAsync(hs, B.st, sizeof(IcpState), cudaMemcpyDeviceToHost, ctx->stream));
  dev_free(ctx, callbuf);
  sync(ctx);
  if (exec) ctx->launches += 5 * static_cast<uint64_t>(hs->launches);  // five kernels per body run
  std::memset(res, 0, sizeof(*res));
  for (int i = 0; i < 16; ++i) {
    res->transform64[i] = hs->T[i];
    res->transform[i] = static_cast<float>(hs->T[i]);
  }
  res->converged = hs->converged;
  res->iterations = hs->iter;
  res->state = hs->state;
  res->n_correspondences = hs->ncorr;
  res->fitness = p->compute_fitness ? hs->fitness : 0.0;
  res->mse = hs->mse;
}
