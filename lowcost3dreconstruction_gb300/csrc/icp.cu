// pcl::IterativeClosestPoint on the GPU (pcl_tools/fine_registration.cpp:105-126).
//
// One launch = one ICP iteration, fused: every warp grabs tiles of 32
// Morton-sorted source points, transforms them by the current FP32 transform,
// finds each point's exact nearest target within the correspondence distance
// (warp-tile traversal), forms the per-correspondence terms in FP32, reduces
// them across the warp with a transposing reduce-scatter (lane l ends with term
// l), and accumulates term l with Kahan compensation in FP32.  Blocks write FP64
// partials; the last block to finish adds them in a fixed order, solves in FP64
// (3x3 SVD for point-to-point, 6x6 LDL^T for point-to-plane), composes and
// re-orthonormalises the transform, applies PCL's DefaultConvergenceCriteria and
// tells the enclosing CUDA-graph WHILE node whether to run another iteration.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "search.cuh"

namespace {

constexpr int kIcpThreads = 256;
constexpr int kIcpWarps = kIcpThreads / 32;

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
};

struct IcpState {
  double T[16];
  Xf Tf;
  double prev_mse, mse, fitness;
  int iter, done, converged, state, ncorr, launches;
  unsigned int tile_ctr, blocks_done;
  unsigned int fit_tile_ctr, fit_blocks_done;
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

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
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

template <int P2PL>
__global__ void __launch_bounds__(kIcpThreads) k_icp_iter(const IcpParams* __restrict__ prm, IcpState* st,
                                                          double* __restrict__ part, cudaGraphConditionalHandle h) {
  __shared__ IndexView s_tgt;
  __shared__ Xf s_T;
  __shared__ WarpScratch wss[kIcpWarps];
  __shared__ double s_acc[kIcpWarps][32];
  __shared__ int s_flag;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_flag = *reinterpret_cast<volatile int*>(&st->done);
    if (s_flag && blockIdx.x == 0 && prm->use_graph) cudaGraphSetConditional(h, 0);
    s_tgt = prm->tgt;
    s_T = st->Tf;
  }
  __syncthreads();
  if (s_flag) return;
  const float4* __restrict__ src = prm->src_pts;
  const int ntiles = prm->src_ntiles;
  const float cap = prm->cap;
  const float c0 = prm->c[0], c1 = prm->c[1], c2 = prm->c[2];
  float acc = 0.f, cmp = 0.f;
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = static_cast<int>(atomicAdd(&st->tile_ctr, 1u));
    tile = __shfl_sync(LCR_FULL, tile, 0);
    if (tile >= ntiles) break;
    const float4 p = src[static_cast<size_t>(tile) * 32 + lane];
    const bool pv = finite3(p.x, p.y, p.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    if (pv) q = xf_apply(s_T, p.x, p.y, p.z);
    float4 tlo, thi;
    if (!tile_box(q.x, q.y, q.z, pv, tlo, thi)) continue;
    NN1 v;
    v.init(q.x, q.y, q.z, pv, cap, tlo, thi);
    tile_traverse(s_tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), wss[wib]);
    float t[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) t[i] = 0.f;
    if (pv && v.found()) {
      const float sx = q.x - c0, sy = q.y - c1, sz = q.z - c2;
      const float tx = v.bp.x - c0, ty = v.bp.y - c1, tz = v.bp.z - c2;
      const float d = key_dist(v.best);
      if (!P2PL) {
        t[0] = sx; t[1] = sy; t[2] = sz;
        t[3] = tx; t[4] = ty; t[5] = tz;
        t[6] = tx * sx; t[7] = tx * sy; t[8] = tx * sz;
        t[9] = ty * sx; t[10] = ty * sy; t[11] = ty * sz;
        t[12] = tz * sx; t[13] = tz * sy; t[14] = tz * sz;
        t[15] = 1.f;
        t[16] = d;
      } else {
        const float4 n = prm->tgt_nrm[key_idx(v.best)];
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
    const float mine = reduce_scatter32(t, lane);
    kahan_add(acc, cmp, mine);
  }
  s_acc[wib][lane] = static_cast<double>(acc) - static_cast<double>(cmp);
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kIcpWarps; ++w) s += s_acc[w][threadIdx.x];
    part[static_cast<size_t>(blockIdx.x) * 32 + threadIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_flag = (atomicAdd(&st->blocks_done, 1u) == gridDim.x - 1) ? 1 : 0;
  __syncthreads();
  if (!s_flag) return;
  __threadfence();
  {  // fixed-order FP64 reduction of the block partials: 8 slices x 32 terms
    const int term = threadIdx.x & 31, slice = threadIdx.x >> 5;
    double s = 0.0;
    for (int b = slice; b < static_cast<int>(gridDim.x); b += kIcpWarps) s += __ldcg(&part[static_cast<size_t>(b) * 32 + term]);
    s_acc[slice][term] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S[32];
    for (int t = 0; t < 32; ++t) {
      double s = 0.0;
      for (int w = 0; w < kIcpWarps; ++w) s += s_acc[w][t];
      S[t] = s;
    }
    icp_update<P2PL>(S, prm, st);
    st->launches += 1;
    if (st->launches > prm->max_iter + 1) st->done = 1;  // hard bound on the device loop
    st->tile_ctr = 0;
    st->blocks_done = 0;
    __threadfence();
    if (prm->use_graph) cudaGraphSetConditional(h, st->done ? 0u : 1u);
  }
}

// getFitnessScore(): mean squared distance from every transformed source point
// to its exact (uncapped) nearest target point.
__global__ void __launch_bounds__(kIcpThreads) k_fitness(const IcpParams* __restrict__ prm, IcpState* st,
                                                         double* __restrict__ part) {
  __shared__ IndexView s_tgt;
  __shared__ Xf s_T;
  __shared__ WarpScratch wss[kIcpWarps];
  __shared__ double s_acc[kIcpWarps][2];
  __shared__ int s_flag;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    s_tgt = prm->tgt;
    s_T = st->Tf;
  }
  __syncthreads();
  const float4* __restrict__ src = prm->src_pts;
  const int ntiles = prm->src_ntiles;
  float acc = 0.f, cmp = 0.f;
  int cnt = 0;
  for (;;) {
    int tile = 0;
    if (lane == 0) tile = static_cast<int>(atomicAdd(&st->fit_tile_ctr, 1u));
    tile = __shfl_sync(LCR_FULL, tile, 0);
    if (tile >= ntiles) break;
    const float4 p = src[static_cast<size_t>(tile) * 32 + lane];
    const bool pv = finite3(p.x, p.y, p.z);
    float3 q = make_float3(0.f, 0.f, 0.f);
    if (pv) q = xf_apply(s_T, p.x, p.y, p.z);
    float4 tlo, thi;
    if (!tile_box(q.x, q.y, q.z, pv, tlo, thi)) continue;
    NN1 v;
    v.init(q.x, q.y, q.z, pv, LCR_INF, tlo, thi);
    tile_traverse(s_tgt, v, 0.5f * (tlo.x + thi.x), 0.5f * (tlo.y + thi.y), 0.5f * (tlo.z + thi.z), wss[wib]);
    if (pv && v.found()) {
      kahan_add(acc, cmp, key_dist(v.best));
      ++cnt;
    }
  }
  double s = static_cast<double>(acc) - static_cast<double>(cmp);
  double c = static_cast<double>(cnt);
  s = warp_sum(s);
  c = warp_sum(c);
  if (lane == 0) {
    s_acc[wib][0] = s;
    s_acc[wib][1] = c;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0.0;
    for (int w = 0; w < kIcpWarps; ++w) t += s_acc[w][threadIdx.x];
    part[static_cast<size_t>(blockIdx.x) * 2 + threadIdx.x] = t;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_flag = (atomicAdd(&st->fit_blocks_done, 1u) == gridDim.x - 1) ? 1 : 0;
  __syncthreads();
  if (!s_flag || threadIdx.x != 0) return;
  __threadfence();
  double ts = 0.0, tc = 0.0;
  for (int b = 0; b < static_cast<int>(gridDim.x); ++b) {
    ts += __ldcg(&part[static_cast<size_t>(b) * 2]);
    tc += __ldcg(&part[static_cast<size_t>(b) * 2 + 1]);
  }
  st->fitness = tc > 0 ? ts / tc : DBL_MAX;
  st->fit_tile_ctr = 0;
  st->fit_blocks_done = 0;
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

int icp_grid(lcr_ctx* ctx) { return ctx->sms * 2; }

// Builds (once per context and method) the graph WHILE(cond) { k_icp_iter }.
// Returns nullptr if conditional nodes are unavailable.
cudaGraphExec_t icp_graph(lcr_ctx* ctx, int p2pl, const IcpBuffers& B) {
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
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaKernelNodeParams kp;
    std::memset(&kp, 0, sizeof(kp));
    kp.func = p2pl ? reinterpret_cast<void*>(k_icp_iter<1>) : reinterpret_cast<void*>(k_icp_iter<0>);
    kp.gridDim = dim3(icp_grid(ctx));
    kp.blockDim = dim3(kIcpThreads);
    kp.sharedMemBytes = 0;
    const IcpParams* a0 = B.prm;
    IcpState* a1 = B.st;
    double* a2 = B.part;
    void* args[] = {&a0, &a1, &a2, &h};
    kp.kernelParams = args;
    cudaGraphNode_t kn = nullptr;
    ok = cudaGraphAddKernelNode(&kn, body, nullptr, 0, &kp) == cudaSuccess;
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
  double c4[4];
  centroid_run(ctx, tgt, c4);
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
  for (int a = 0; a < 3; ++a) hp->c[a] = static_cast<float>(c4[a]);
  hp->min_corr = 3;
  hp->max_iter = p->max_iterations;
  hp->teps = p->transformation_epsilon;
  hp->feps = p->euclidean_fitness_epsilon;
  hp->use_graph = exec ? 1 : 0;
  const double I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  for (int i = 0; i < 16; ++i) hs->T[i] = guess ? static_cast<double>(guess[i]) : I[i];
  for (int i = 0; i < 12; ++i) hs->Tf.m[i] = static_cast<float>(hs->T[i]);
  hs->prev_mse = DBL_MAX;
  CUDA_TRY(cudaMemcpyAsync(B.prm, stage, 2048, cudaMemcpyHostToDevice, ctx->stream));

  if (exec) {
    CUDA_TRY(cudaGraphLaunch(exec, ctx->stream));
  } else {
    cudaGraphConditionalHandle none = 0;
    for (int it = 0; it < p->max_iterations; ++it) {
      if (p2pl) LCR_LAUNCH(ctx, k_icp_iter<1>, grid, kIcpThreads, 0, B.prm, B.st, B.part, none);
      else LCR_LAUNCH(ctx, k_icp_iter<0>, grid, kIcpThreads, 0, B.prm, B.st, B.part, none);
      if ((it & 7) == 7) {
        int* hd = static_cast<int*>(pinned(ctx, 2048)) + 384;
        CUDA_TRY(cudaMemcpyAsync(hd, &B.st->done, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        if (*hd) break;
      }
    }
  }
  if (p->compute_fitness) LCR_LAUNCH(ctx, k_fitness, grid, kIcpThreads, 0, B.prm, B.st, B.part);
  CUDA_TRY(cudaMemcpyAsync(hs, B.st, sizeof(IcpState), cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  if (exec) ctx->launches += static_cast<uint64_t>(hs->launches);
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
