// Super-resolution front end of the captures (capture/super_resolution/
// super_resolution.cpp:236-314): a burst of F depth frames of one view is
// registered to its first frame, warped onto it, upsampled, fused by the
// zero-eliminated mean and resampled back to the sensor grid.
//
//  1. observed min / max over the nonzero pixels of the burst      :236-252
//  2. ECC affine registration of every frame to frame 0            :255-260
//     (enhanced correlation coefficient maximisation, Evangelidis &
//     Psarakis 2008, as cv::findTransformECC with MOTION_AFFINE: both
//     images smoothed by a 5x5 Gaussian (sigma 1.1), central-difference
//     gradients, Gauss-Newton steps on the correlation coefficient, stop
//     when it changes by less than eps or after the iteration limit)
//  3. inverse-map affine warp of frames 1.. (bilinear, zero outside) :267-270
//  4. nearest upsampling by the factor and the ZE-mean per pixel     :274-310
//  5. Lanczos-4 resampling back to the sensor grid, rounded and
//     saturated to uint16                                           :312-314
// The Kinect v2 form (super_resolution_kv2.cpp:222-311) takes float frames,
// leaves an uncovered pixel at 0 and returns the float result unrounded.
//
// All frames of a burst register at once: one pass per iteration accumulates
// for every frame the 45 sums the Gauss-Newton step needs (FP32 pairs: exact
// to ~2^-44 for the correlation coefficient, Kahan-compensated for the
// Jacobian terms, added in a fixed order), and the last block of each frame
// takes the FP64 step on one thread.
// The smoothing and gradient filters mirror the border at its edge pixel
// (reflect-101); the Lanczos taps clamp to the image.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "lcr_internal.cuh"

namespace {

constexpr int kSums = 45;  // n, SI, SII, ST, STT, SIT, SJ[6], SJI[6], SJT[6], SJJ[21]

__device__ __forceinline__ int reflect101(int i, int n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
  return i;
}

// Frames to float, and the range of the positive values (as their bit
// patterns, which order positive floats as their values): per-thread over a
// grid-stride loop, then warp and block reductions, one atomic pair per block
// (a pair per warp contends on the two words).
__device__ __forceinline__ unsigned range_key(uint16_t v) { return v; }
__device__ __forceinline__ unsigned range_key(float v) { return __float_as_uint(v); }

template <typename T>
__global__ void k_sr_float(const T* __restrict__ in, size_t n, float* __restrict__ out,
                           unsigned int* __restrict__ minmax) {
  unsigned lo = 0xffffffffu, hi = 0u;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const T v = in[i];
    out[i] = static_cast<float>(v);
    if (v > 0) {
      lo = min(lo, range_key(v));
      hi = max(hi, range_key(v));
    }
  }
  lo = __reduce_min_sync(LCR_FULL, lo);
  hi = __reduce_max_sync(LCR_FULL, hi);
  __shared__ unsigned slo[32], shi[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) {
    slo[wid] = lo;
    shi[wid] = hi;
  }
  __syncthreads();
  if (wid == 0) {
    lo = lane < nw ? slo[lane] : 0xffffffffu;
    hi = lane < nw ? shi[lane] : 0u;
    lo = __reduce_min_sync(LCR_FULL, lo);
    hi = __reduce_max_sync(LCR_FULL, hi);
    if (lane == 0 && hi > 0) {
      atomicMin(&minmax[0], lo);
      atomicMax(&minmax[1], hi);
    }
  }
}

// Separable 5-tap Gaussian (weights g[0..2] for offsets 0, 1, 2), horizontal
// then vertical, reflect-101 borders; one frame per blockIdx.z.
__global__ void k_sr_blur_h(const float* __restrict__ in, int w, int h, float g0, float g1, float g2,
                            float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const float* r = in + (static_cast<size_t>(blockIdx.z) * h + y) * w;
  float s = g0 * r[x];
  s += g1 * (r[reflect101(x - 1, w)] + r[reflect101(x + 1, w)]);
  s += g2 * (r[reflect101(x - 2, w)] + r[reflect101(x + 2, w)]);
  out[(static_cast<size_t>(blockIdx.z) * h + y) * w + x] = s;
}

__global__ void k_sr_blur_v(const float* __restrict__ in, int w, int h, float g0, float g1, float g2,
                            float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const float* f = in + static_cast<size_t>(blockIdx.z) * h * w;
  auto at = [&](int yy) { return f[static_cast<size_t>(reflect101(yy, h)) * w + x]; };
  float s = g0 * at(y);
  s += g1 * (at(y - 1) + at(y + 1));
  s += g2 * (at(y - 2) + at(y + 2));
  out[(static_cast<size_t>(blockIdx.z) * h + y) * w + x] = s;
}

// Central differences 0.5 (f(x+1) - f(x-1)), reflect-101 borders, packed with
// the smoothed value as (value, d/dx, d/dy, 0): the registration reads all
// three at each bilinear tap with one 16-byte load.
__global__ void k_sr_grad(const float* __restrict__ in, int w, int h, float4* __restrict__ pk) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const float* f = in + static_cast<size_t>(blockIdx.z) * h * w;
  const size_t o = (static_cast<size_t>(blockIdx.z) * h + y) * w + x;
  const float gx = 0.5f * (f[static_cast<size_t>(y) * w + reflect101(x + 1, w)] - f[static_cast<size_t>(y) * w + reflect101(x - 1, w)]);
  const float gy = 0.5f * (f[static_cast<size_t>(reflect101(y + 1, h)) * w + x] - f[static_cast<size_t>(reflect101(y - 1, h)) * w + x]);
  pk[o] = make_float4(f[static_cast<size_t>(y) * w + x], gx, gy, 0.f);
}

// Bilinear sample with a zero border: a tap outside the image contributes 0.
__device__ __forceinline__ float bilinear(const float* __restrict__ f, int w, int h, float u, float v) {
  const float fu = floorf(u), fv = floorf(v);
  const int x0 = static_cast<int>(fu), y0 = static_cast<int>(fv);
  const float ax = u - fu, ay = v - fv;
  auto at = [&](int xx, int yy) {
    return (xx >= 0 && yy >= 0 && xx < w && yy < h) ? f[static_cast<size_t>(yy) * w + xx] : 0.f;
  };
  const float top = at(x0, y0) * (1.f - ax) + at(x0 + 1, y0) * ax;
  const float bot = at(x0, y0 + 1) * (1.f - ax) + at(x0 + 1, y0 + 1) * ax;
  return top * (1.f - ay) + bot * ay;
}

// (a.x + a.y) + (b.x + b.y) as a pair of FP32 values: the exact two-sum of
// the leading parts, the trailing parts and its error renormalised into the
// pair (about 44 significant bits for sums of like-signed terms).
__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {
  const float sum = __fadd_rn(a.x, b.x), bp = __fsub_rn(sum, a.x);
  const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(sum, bp)), __fsub_rn(b.x, bp));
  const float l = __fadd_rn(__fadd_rn(a.y, b.y), e);
  const float hi = __fadd_rn(sum, l);
  return make_float2(hi, __fsub_rn(l, __fsub_rn(hi, sum)));
}

// Solves H x1 = b1 and H x2 = b2 for the symmetric positive definite 6x6
// Gauss-Newton matrix H = sum J^T J by one LDL^T factorisation (FP64, no
// square roots, one reciprocal per pivot, every index fixed at compile time
// so that it all stays in registers: FP64 latency is what bounds this
// single-thread step); false when H is not positive definite.
__device__ __forceinline__ bool ldl_solve6(const double H[6][6], const double b1[6], const double b2[6],
                                           double x1[6], double x2[6]) {
  double L[6][6], E[6][6], dinv[6];  // L unit lower triangular, E = L D
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = H[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= E[j][k] * L[j][k];
    if (!(d > 0.0)) return false;
    dinv[j] = 1.0 / d;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double t = H[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) t -= E[i][k] * L[j][k];
      E[i][j] = t;
      L[i][j] = t * dinv[j];
    }
  }
  double y1[6], y2[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double t1 = b1[i], t2 = b2[i];
#pragma unroll
    for (int k = 0; k < i; ++k) {
      t1 -= L[i][k] * y1[k];
      t2 -= L[i][k] * y2[k];
    }
    y1[i] = t1;
    y2[i] = t2;
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    double t1 = y1[i] * dinv[i], t2 = y2[i] * dinv[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) {
      t1 -= L[k][i] * x1[k];
      t2 -= L[k][i] * x2[k];
    }
    x1[i] = t1;
    x2[i] = t2;
  }
  return true;
}

// The ECC step of frame f from its 45 sums: correlation coefficient, the
// Gauss-Newton update of the warp, the stopping tests (iteration limit,
// |rho - rho_prev| < eps, a singular system, no improvement along the step).
__device__ void ecc_step(const double* s, int f, float* warps, double* rho, int* active, int* iters, double eps,
                         int max_iter) {
  const double n = s[0];
  iters[f] += 1;
  if (!(n > 0.0)) {
    active[f] = 0;
    return;
  }
  const double inv_n = 1.0 / n, mi = s[1] * inv_n, mt = s[3] * inv_n;
  const double img_var = s[2] - n * mi * mi, tmp_var = s[4] - n * mt * mt;
  const double corr = s[5] - mi * s[3] - mt * s[1] + n * mi * mt;
  const double r = img_var > 0.0 && tmp_var > 0.0 ? corr * rsqrt(img_var * tmp_var) : 0.0;
  double ip[6], tp[6], H[6][6];
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    ip[a] = s[12 + a] - mi * s[6 + a];
    tp[a] = s[18 + a] - mt * s[6 + a];
  }
  int q = 24;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = a; b < 6; ++b) H[a][b] = H[b][a] = s[q++];
  double hi[6], ht[6];  // H^-1 ip and H^-1 tp
  if (!ldl_solve6(H, ip, tp, hi, ht)) {
    active[f] = 0;
    return;
  }
  double lam_n = img_var, lam_d = corr;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    lam_n -= ip[a] * hi[a];
    lam_d -= tp[a] * hi[a];
  }
  if (!(lam_d > 0.0)) {  // the correlation did not improve along the step: stop (the cv routine fails here)
    active[f] = 0;
    return;
  }
  const double lam = lam_n / lam_d;
  // deltaP = H^-1 (lam tp - ip) = lam ht - hi
  double dp[6];
#pragma unroll
  for (int a = 0; a < 6; ++a) dp[a] = lam * ht[a] - hi[a];
  float* m = warps + 6 * f;
  m[0] += static_cast<float>(dp[0]);
  m[3] += static_cast<float>(dp[1]);
  m[1] += static_cast<float>(dp[2]);
  m[4] += static_cast<float>(dp[3]);
  m[2] += static_cast<float>(dp[4]);
  m[5] += static_cast<float>(dp[5]);
  const double prev = rho[f];
  rho[f] = r;
  if (fabs(r - prev) < eps || iters[f] >= max_iter) active[f] = 0;
}

// One ECC pass for frame f = list[blockIdx.y] (the frames still iterating),
// blockIdx.x striding over the pixels: per template pixel (x, y) the
// input sampled at W(x, y) = (m0 x + m1 y + m2, m3 x + m4 y + m5), its
// gradients, the validity mask (all four bilinear taps inside the image: a
// half-outside sample of a depth image is a large outlier) and the masked
// Jacobian J = (x gx, x gy, y gx, y gy, gx, gy) with respect to
// (m0, m3, m1, m4, m2, m5); the block's 45 sums go to part[frame][block][45].
constexpr int kEccThreads = 256;
__global__ void __launch_bounds__(kEccThreads, 2)
    k_ecc_pass(const float4* __restrict__ pk, int w, int h, const int* __restrict__ list, float* warps, int* active,
               float2* part, unsigned int* done, double* rho, int* iters, double eps, int max_iter) {
  const int f = list[blockIdx.y];
  if (!active[f]) return;
  __shared__ float2 red[kEccThreads / 32][kSums];
  const float m[6] = {warps[6 * f], warps[6 * f + 1], warps[6 * f + 2],
                      warps[6 * f + 3], warps[6 * f + 4], warps[6 * f + 5]};
  const size_t plane = static_cast<size_t>(w) * h;
  const float4* P = pk + f * plane;  // frame f: (smoothed, d/dx, d/dy, 0) per pixel
  // Every sum is kept as an unevaluated pair hi + lo of FP32 values (FP32
  // pipes only: the FP64 ones are a small fraction of them on this part).
  // The five sums of the correlation coefficient are exact to ~2^-44: the
  // products split exactly by an FMA (p + e = a b), p added by an exact
  // two-sum, the errors collected in lo.  The coefficient's change is the
  // stopping test, and FP32 rounding of I^2 at depths near 1000 would leave
  // it jittering by ~1e-8 between iterations, so the iteration would never
  // stop at eps ~1e-12.  The 39 Jacobian sums take FP32 products with Kahan
  // compensation.  Pairs are added across the warp by the same two-sum and
  // widened to FP64 for the block and grid reductions.
  int rn = 0;
  float rh[5], rl[5];  // SI, SII, ST, STT, SIT
  float ks[kSums - 6], kc[kSums - 6];
#pragma unroll
  for (int k = 0; k < 5; ++k) rh[k] = rl[k] = 0.f;
#pragma unroll
  for (int k = 0; k < kSums - 6; ++k) ks[k] = kc[k] = 0.f;
  auto exact_add = [&](int k, float a, float b) {  // rh/rl[k] += a * b, b == 1 for a plain term
    const float pp = __fmul_rn(a, b), pe = __fmaf_rn(a, b, -pp);
    const float sum = __fadd_rn(rh[k], pp), bp = __fsub_rn(sum, rh[k]);
    const float e = __fadd_rn(__fsub_rn(rh[k], __fsub_rn(sum, bp)), __fsub_rn(pp, bp));
    rh[k] = sum;
    rl[k] = __fadd_rn(rl[k], __fadd_rn(e, pe));
  };
  const int npix = w * h;
  const int stride = gridDim.x * kEccThreads, sy = stride / w, sx = stride - sy * w;
  int p = blockIdx.x * kEccThreads + threadIdx.x, y = p / w, x = p - y * w;
  for (; p < npix; p += stride, x += sx, y += sy) {
    if (x >= w) {
      x -= w;
      ++y;
    }
    const float u = m[0] * x + m[1] * y + m[2], v = m[3] * x + m[4] * y + m[5];
    const float fu = floorf(u), fv = floorf(v);
    if (!(fu >= 0.f && fv >= 0.f && fu + 1.f < w && fv + 1.f < h)) continue;  // outside the mask: no terms
    // all four taps are inside: the zero-border bilinear sample without its checks
    const int x0 = static_cast<int>(fu), y0 = static_cast<int>(fv);
    const float ax = u - fu, ay = v - fv;
    const float4* r0 = P + static_cast<size_t>(y0) * w + x0;
    const float4 a = r0[0], b = r0[1], c = r0[w], d = r0[w + 1];
    auto lerp2 = [&](float va, float vb, float vc, float vd) {
      const float top = va * (1.f - ax) + vb * ax;
      const float bot = vc * (1.f - ax) + vd * ax;
      return top * (1.f - ay) + bot * ay;
    };
    const float iw = lerp2(a.x, b.x, c.x, d.x), gx = lerp2(a.y, b.y, c.y, d.y), gy = lerp2(a.z, b.z, c.z, d.z);
    const float t = pk[p].x;
    rn += 1;
    exact_add(0, iw, 1.f);
    exact_add(1, iw, iw);
    exact_add(2, t, 1.f);
    exact_add(3, t, t);
    exact_add(4, iw, t);
    const float fx = static_cast<float>(x), fy = static_cast<float>(y);
    const float J[6] = {fx * gx, fx * gy, fy * gx, fy * gy, gx, gy};
    auto kadd = [&](int k, float val) {
      const float yk = val - kc[k];
      const float tk = ks[k] + yk;
      kc[k] = (tk - ks[k]) - yk;
      ks[k] = tk;
    };
    int q = 18;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      kadd(a, J[a]);
      kadd(6 + a, J[a] * iw);
      kadd(12 + a, J[a] * t);
#pragma unroll
      for (int b = a; b < 6; ++b) kadd(q++, J[a] * J[b]);
    }
  }
  // The warp's 45 pairs (padded to 48) by a reduce-scatter: at offsets 16, 8,
  // 4, 2 each lane keeps the half of its values that its lane bit selects and
  // adds the partner's copy of that half (48 pair additions per lane instead
  // of 5 x 45 for a butterfly per sum); offset 1 is a butterfly on the last
  // three.  Lane l then holds sums 24 b4 + 12 b3 + 6 b2 + 3 b1 + 0..2 of the
  // warp, b the bits of l.
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2 v[48];
#pragma unroll
  for (int k = 0; k < 48; ++k)
    v[k] = k == 0 ? make_float2(static_cast<float>(rn), 0.f)
         : k <= 5 ? make_float2(rh[k - 1], rl[k - 1])
         : k < kSums ? make_float2(ks[k - 6], -kc[k - 6]) : make_float2(0.f, 0.f);
  auto halve = [&](int n, int o) {  // v[0..2n) -> v[0..n)
    const bool upper = lane & o;
#pragma unroll
    for (int j = 0; j < 24; ++j) {
      if (j < n) {
        const float2 keep = upper ? v[n + j] : v[j], send = upper ? v[j] : v[n + j];
        const float2 got = make_float2(__shfl_xor_sync(LCR_FULL, send.x, o), __shfl_xor_sync(LCR_FULL, send.y, o));
        v[j] = pair_add(keep, got);
      }
    }
  };
  halve(24, 16);
  halve(12, 8);
  halve(6, 4);
  halve(3, 2);
#pragma unroll
  for (int j = 0; j < 3; ++j)
    v[j] = pair_add(v[j], make_float2(__shfl_xor_sync(LCR_FULL, v[j].x, 1), __shfl_xor_sync(LCR_FULL, v[j].y, 1)));
  if (!(lane & 1)) {
    const int base = (lane & 16 ? 24 : 0) + (lane & 8 ? 12 : 0) + (lane & 4 ? 6 : 0) + (lane & 2 ? 3 : 0);
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (base + j < kSums) red[wid][base + j] = v[j];
  }
  __syncthreads();
  if (threadIdx.x < kSums) {
    float2 v = red[0][threadIdx.x];
#pragma unroll
    for (int j = 1; j < kEccThreads / 32; ++j) v = pair_add(v, red[j][threadIdx.x]);
    part[(static_cast<size_t>(f) * gridDim.x + blockIdx.x) * kSums + threadIdx.x] = v;
  }
  // The last block of the frame to finish adds the blocks' sums in a fixed
  // order (warp j takes blocks j, j + 8, ...; then the warps in order) and
  // takes the step; every block has read the warp before it counts itself,
  // so the update races with no reader.
  __shared__ bool last;
  __shared__ double total[kSums];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&done[f], 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const float2* pp = part + static_cast<size_t>(f) * gridDim.x * kSums;
  for (int k = lane; k < kSums; k += 32) {
    float2 v = make_float2(0.f, 0.f);
#pragma unroll 8
    for (unsigned bk = wid; bk < gridDim.x; bk += kEccThreads / 32)
      v = pair_add(v, __ldcg(pp + static_cast<size_t>(bk) * kSums + k));
    red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < kSums) {
    float2 v = red[0][threadIdx.x];
#pragma unroll
    for (int j = 1; j < kEccThreads / 32; ++j) v = pair_add(v, red[j][threadIdx.x]);
    total[threadIdx.x] = static_cast<double>(v.x) + static_cast<double>(v.y);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    done[f] = 0;
    ecc_step(total, f, warps, rho, active, iters, eps, max_iter);
  }
}

// ZE-mean on the sensor grid (nearest upsampling by the factor commutes with
// it, so the high-resolution image is never formed): ze(y, x) is the mean of
// the positive values among frame 0 at (x, y) and frames k >= 1 sampled at
// W_k(x, y) (the inverse-map bilinear warp, zero outside); FP64 sum in frame
// order divided by the count, to float; a pixel with no positive value is
// 0/0 = NaN (super_resolution.cpp's mean of an empty vector) or, with
// empty_zero, 0 (super_resolution_kv2.cpp:298 skips it; its output buffer is
// uninitialised there, and 0 stands for that).
__global__ void k_sr_fuse(const float* __restrict__ in, int w, int h, int F, const float* __restrict__ warps,
                          int empty_zero, float* __restrict__ ze) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const size_t plane = static_cast<size_t>(w) * h, o = static_cast<size_t>(y) * w + x;
  double sum = 0.0;
  int cnt = 0;
  for (int f = 0; f < F; ++f) {
    const float* m = warps + 6 * f;
    const float v = f == 0 ? in[o] : bilinear(in + f * plane, w, h, m[0] * x + m[1] * y + m[2], m[3] * x + m[4] * y + m[5]);
    if (v > 0.f) {
      sum += v;
      ++cnt;
    }
  }
  ze[o] = cnt == 0 && empty_zero ? 0.f : static_cast<float>(sum / cnt);
}

// Lanczos-4 resampling of the upsampled image by 1/s, one axis per pass:
// output o reads the 8 upsampled samples base[o] .. base[o] + 7 (clamped to
// the upsampled extent) with weights wgt[o][0..7]; upsampled sample X is
// sensor sample X / s.  The horizontal pass runs on the h distinct rows.
__global__ void k_sr_lanczos_h(const float* __restrict__ ze, int w, int s, const int* __restrict__ base,
                               const float* __restrict__ wgt, float* __restrict__ half) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const int W = w * s;
  const float* row = ze + static_cast<size_t>(y) * w;
  float acc = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) acc += wgt[8 * x + i] * row[min(max(base[x] + i, 0), W - 1) / s];
  half[static_cast<size_t>(y) * w + x] = acc;
}

// The vertical pass; uint16 output is rounded half to even and saturated
// (NaN -> 0), float output is the value itself.
__device__ __forceinline__ void store_depth(uint16_t* out, float v) {
  float r = rintf(v);
  if (!(r > 0.f)) r = 0.f;
  if (r > 65535.f) r = 65535.f;
  *out = static_cast<uint16_t>(r);
}
__device__ __forceinline__ void store_depth(float* out, float v) { *out = v; }

template <typename T>
__global__ void k_sr_lanczos_v(const float* __restrict__ half, int w, int h, int s, const int* __restrict__ base,
                               const float* __restrict__ wgt, T* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const int H = h * s;
  float acc = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) acc += wgt[8 * y + i] * half[static_cast<size_t>(min(max(base[y] + i, 0), H - 1) / s) * w + x];
  store_depth(out + static_cast<size_t>(y) * w + x, acc);
}

// Lanczos (a = 4) taps of output o = 0 .. n - 1 of a resampling by 1/s: the
// source position p = (o + 0.5) s - 0.5 (exact in binary), taps floor(p) - 3
// .. floor(p) + 4 with weights L(d) = sinc(d) sinc(d / 4), normalised to sum
// 1; a whole p takes the centre tap alone.
void lanczos_table(int n, int s, int* base, float* wgt) {
  const double pi = 3.14159265358979323846;
  for (int o = 0; o < n; ++o) {
    const double p = (o + 0.5) * s - 0.5, fl = std::floor(p), t = static_cast<float>(p - fl);
    base[o] = static_cast<int>(fl) - 3;
    float* wo = wgt + 8 * o;
    if (t < 1.1920929e-7) {
      for (int i = 0; i < 8; ++i) wo[i] = i == 3 ? 1.f : 0.f;
      continue;
    }
    double sum = 0.0, ww[8];
    for (int i = 0; i < 8; ++i) {
      const double a = pi * ((i - 3) - t);
      ww[i] = 4.0 * std::sin(a) * std::sin(a / 4.0) / (a * a);
      sum += ww[i];
    }
    for (int i = 0; i < 8; ++i) wo[i] = static_cast<float>(ww[i] / sum);
  }
}

}  // namespace

void super_resolve_run(lcr_ctx* ctx, const void* frames, bool f32, int w, int h, int F, int factor, int max_iter,
                       double eps, void* out, float* warps_out, float minmax_out[2], int* iters_out) {
  const size_t esz = f32 ? 4 : 2;
  const size_t plane = static_cast<size_t>(w) * h, all = plane * F;
  // The pass runs one wave of resident blocks, shared among the frames still
  // iterating (the others return at once): many pixels per thread while all
  // frames register, the whole GPU on the last one.
  int per_sm = 1;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ecc_pass, kEccThreads, 0));
  const int resident = std::max(1, per_sm) * ctx->sms;
  const int nblocks = std::max(1, std::min(resident, static_cast<int>((plane + kEccThreads - 1) / kEccThreads)));
  const size_t table = static_cast<size_t>(w + h) * 9 * 4;
  const size_t bytes = all * 4 + 3 * all * 4 + all * 16 + 2 * plane * 4 + plane * 4 + table + F * (24 + 8 + 8 + 4) +
                       static_cast<size_t>(F) * nblocks * kSums * 8 + 64;
  char* blk = static_cast<char*>(dev_alloc(ctx, bytes + 32 * 256));  // every take() below pads to 256
  char* q = blk;
  auto take = [&](size_t b) {
    char* r = q;
    q += (b + 255) & ~static_cast<size_t>(255);
    return r;
  };
  void* din = take(all * esz);
  auto* img = reinterpret_cast<float*>(take(all * 4));
  auto* tmp = reinterpret_cast<float*>(take(all * 4));
  auto* blur = reinterpret_cast<float*>(take(all * 4));
  auto* pk = reinterpret_cast<float4*>(take(all * 16));
  auto* ze = reinterpret_cast<float*>(take(plane * 4));
  auto* half = reinterpret_cast<float*>(take(plane * 4));
  auto* tab = take(table);
  void* dout = take(plane * esz);
  auto* warps = reinterpret_cast<float*>(take(F * 24));
  auto* rho = reinterpret_cast<double*>(take(F * 8));
  auto* active = reinterpret_cast<int*>(take(F * 4));
  auto* iters = reinterpret_cast<int*>(take(F * 4));
  auto* done = reinterpret_cast<unsigned int*>(take(F * 4));
  auto* list = reinterpret_cast<int*>(take(F * 4));
  auto* part = reinterpret_cast<float2*>(take(static_cast<size_t>(F) * nblocks * kSums * 8));
  auto* flags = reinterpret_cast<unsigned int*>(take(64));
  CUDA_TRY(cudaMemcpyAsync(din, frames, all * esz, cudaMemcpyHostToDevice, ctx->stream));
  const unsigned int init[3] = {0xffffffffu, 0u, 0u};
  CUDA_TRY(cudaMemcpyAsync(flags, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
  const unsigned gconv = static_cast<unsigned>(std::min<size_t>((all + 255) / 256, 4 * ctx->sms));
  if (f32)
    LCR_LAUNCH(ctx, k_sr_float<float>, gconv, 256, 0, static_cast<const float*>(din), all, img, flags);
  else
    LCR_LAUNCH(ctx, k_sr_float<uint16_t>, gconv, 256, 0, static_cast<const uint16_t*>(din), all, img, flags);
  // 5x5 Gaussian, sigma 0.3 ((5 - 1) / 2 - 1) + 0.8 = 1.1
  const double sg = 1.1;
  double g[3] = {1.0, std::exp(-1.0 / (2 * sg * sg)), std::exp(-4.0 / (2 * sg * sg))};
  const double gs = g[0] + 2 * g[1] + 2 * g[2];
  const float g0 = static_cast<float>(g[0] / gs), g1 = static_cast<float>(g[1] / gs), g2 = static_cast<float>(g[2] / gs);
  const dim3 gimg((w + 127) / 128, h, F);
  LCR_LAUNCH(ctx, k_sr_blur_h, gimg, 128, 0, img, w, h, g0, g1, g2, tmp);
  LCR_LAUNCH(ctx, k_sr_blur_v, gimg, 128, 0, tmp, w, h, g0, g1, g2, blur);
  LCR_LAUNCH(ctx, k_sr_grad, gimg, 128, 0, blur, w, h, pk);
  std::vector<float> hw(6 * F, 0.f);
  for (int f = 0; f < F; ++f) {
    hw[6 * f + 0] = 1.f;
    hw[6 * f + 4] = 1.f;
  }
  std::vector<int> hact(F, 1);
  hact[0] = 0;
  std::vector<double> hrho(F, -1.0);
  CUDA_TRY(cudaMemcpyAsync(warps, hw.data(), F * 24, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(active, hact.data(), F * 4, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(rho, hrho.data(), F * 8, cudaMemcpyHostToDevice, ctx->stream));
  CUDA_TRY(cudaMemsetAsync(iters, 0, F * 4, ctx->stream));
  CUDA_TRY(cudaMemsetAsync(done, 0, F * 4, ctx->stream));
  // The host reads which frames are still iterating after 2, 4, 8, ... 32
  // iterations and every 32 after that; the next iterations' wave of blocks
  // is shared among those frames alone (blockIdx.y indexes their list), and
  // a frame that stops within a chunk costs its blocks an early return.
  std::vector<int> hlist;
  for (int f = 1; f < F; ++f) hlist.push_back(f);
  for (int it = 0, chunk = 2; it < max_iter && !hlist.empty(); chunk = std::min(2 * chunk, 32)) {
    const int na = static_cast<int>(hlist.size()), nb = std::max(1, nblocks / na);
    CUDA_TRY(cudaMemcpyAsync(list, hlist.data(), na * 4, cudaMemcpyHostToDevice, ctx->stream));
    const int todo = std::min(chunk, max_iter - it);
    for (int k = 0; k < todo; ++k, ++it)
      LCR_LAUNCH(ctx, k_ecc_pass, dim3(nb, na), kEccThreads, 0, pk, w, h, list, warps, active, part, done, rho, iters,
                 eps, max_iter);
    CUDA_TRY(cudaMemcpyAsync(hact.data(), active, F * 4, cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
    hlist.clear();
    for (int f = 1; f < F; ++f)
      if (hact[f]) hlist.push_back(f);
  }
  std::vector<char> htab(table);
  auto* xbase = reinterpret_cast<int*>(htab.data());
  auto* ybase = xbase + w;
  auto* xw = reinterpret_cast<float*>(ybase + h);
  auto* yw = xw + 8 * w;
  lanczos_table(w, factor, xbase, xw);
  lanczos_table(h, factor, ybase, yw);
  CUDA_TRY(cudaMemcpyAsync(tab, htab.data(), table, cudaMemcpyHostToDevice, ctx->stream));
  const auto* dxbase = reinterpret_cast<const int*>(tab);
  const auto* dybase = dxbase + w;
  const auto* dxw = reinterpret_cast<const float*>(dybase + h);
  const auto* dyw = dxw + 8 * w;
  const dim3 grow((w + 127) / 128, h);
  LCR_LAUNCH(ctx, k_sr_fuse, grow, 128, 0, img, w, h, F, warps, f32 ? 1 : 0, ze);
  LCR_LAUNCH(ctx, k_sr_lanczos_h, grow, 128, 0, ze, w, factor, dxbase, dxw, half);
  if (f32)
    LCR_LAUNCH(ctx, k_sr_lanczos_v<float>, grow, 128, 0, half, w, h, factor, dybase, dyw, static_cast<float*>(dout));
  else
    LCR_LAUNCH(ctx, k_sr_lanczos_v<uint16_t>, grow, 128, 0, half, w, h, factor, dybase, dyw,
               static_cast<uint16_t*>(dout));
  CUDA_TRY(cudaMemcpyAsync(out, dout, plane * esz, cudaMemcpyDeviceToHost, ctx->stream));
  if (warps_out) CUDA_TRY(cudaMemcpyAsync(warps_out, warps, F * 24, cudaMemcpyDeviceToHost, ctx->stream));
  if (iters_out) CUDA_TRY(cudaMemcpyAsync(iters_out, iters, F * 4, cudaMemcpyDeviceToHost, ctx->stream));
  unsigned int mm[2];
  CUDA_TRY(cudaMemcpyAsync(mm, flags, 8, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  if (minmax_out) {
    auto value = [&](unsigned k) {
      if (!f32) return static_cast<float>(k);
      float v;
      std::memcpy(&v, &k, 4);
      return v;
    };
    minmax_out[0] = mm[1] ? value(mm[0]) : 0.f;
    minmax_out[1] = mm[1] ? value(mm[1]) : 0.f;
  }
  dev_free(ctx, blk);
}
