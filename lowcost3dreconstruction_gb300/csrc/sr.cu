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
//
// All frames of a burst register at once: one pass per iteration accumulates
// for every frame the 45 sums the Gauss-Newton step needs (FP32 products,
// FP64 sums in a fixed order), and one thread per frame solves the 6x6 system.
// The smoothing and gradient filters mirror the border at its edge pixel
// (reflect-101); the Lanczos taps clamp to the image.
#include <cmath>
#include <vector>

#include "lcr_internal.cuh"

namespace {

constexpr int kSums = 45;  // n, SI, SII, ST, STT, SIT, SJ[6], SJI[6], SJT[6], SJJ[21]

__device__ __forceinline__ int reflect101(int i, int n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
  return i;
}

__global__ void k_sr_float(const uint16_t* __restrict__ in, size_t n, float* __restrict__ out,
                           unsigned int* __restrict__ minmax) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint16_t v = in[i];
  out[i] = static_cast<float>(v);
  if (v > 0) {
    atomicMin(&minmax[0], v);
    atomicMax(&minmax[1], v);
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

// Central differences 0.5 (f(x+1) - f(x-1)), reflect-101 borders.
__global__ void k_sr_grad(const float* __restrict__ in, int w, int h, float* __restrict__ gx,
                          float* __restrict__ gy) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= w) return;
  const float* f = in + static_cast<size_t>(blockIdx.z) * h * w;
  const size_t o = (static_cast<size_t>(blockIdx.z) * h + y) * w + x;
  gx[o] = 0.5f * (f[static_cast<size_t>(y) * w + reflect101(x + 1, w)] - f[static_cast<size_t>(y) * w + reflect101(x - 1, w)]);
  gy[o] = 0.5f * (f[static_cast<size_t>(reflect101(y + 1, h)) * w + x] - f[static_cast<size_t>(reflect101(y - 1, h)) * w + x]);
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

// One ECC pass for frame f = 1 + blockIdx.y: per template pixel (x, y) the
// input sampled at W(x, y) = (m0 x + m1 y + m2, m3 x + m4 y + m5), its
// gradients, the validity mask (all four bilinear taps inside the image: a
// half-outside sample of a depth image is a large outlier) and the masked
// Jacobian J = (x gx, x gy, y gx, y gy, gx, gy) with respect to
// (m0, m3, m1, m4, m2, m5); the block's 45 sums go to part[frame][block][45].
constexpr int kEccThreads = 256;
__global__ void __launch_bounds__(kEccThreads) k_ecc_pass(const float* __restrict__ tmpl, const float* __restrict__ img,
                                                           const float* __restrict__ gxs, const float* __restrict__ gys,
                                                           int w, int h, const float* __restrict__ warps,
                                                           const int* __restrict__ active, double* __restrict__ part) {
  const int f = 1 + blockIdx.y;
  if (!active[f]) return;
  __shared__ double red[kEccThreads / 32][kSums];
  const float* m = warps + 6 * f;
  const size_t plane = static_cast<size_t>(w) * h;
  const float* I = img + f * plane;
  const float* GX = gxs + f * plane;
  const float* GY = gys + f * plane;
  double acc[kSums];
#pragma unroll
  for (int k = 0; k < kSums; ++k) acc[k] = 0.0;
  const int npix = w * h;
  for (int p = blockIdx.x * kEccThreads + threadIdx.x; p < npix; p += gridDim.x * kEccThreads) {
    const int x = p % w, y = p / w;
    const float u = m[0] * x + m[1] * y + m[2], v = m[3] * x + m[4] * y + m[5];
    const float iw = bilinear(I, w, h, u, v), gx = bilinear(GX, w, h, u, v), gy = bilinear(GY, w, h, u, v);
    const float fu = floorf(u), fv = floorf(v);
    const float mk = (fu >= 0.f && fv >= 0.f && fu + 1.f < w && fv + 1.f < h) ? 1.f : 0.f;
    const float t = tmpl[p];
    const float J[6] = {mk * x * gx, mk * x * gy, mk * y * gx, mk * y * gy, mk * gx, mk * gy};
    const float mi = mk * iw, mt = mk * t;
    acc[0] += mk;
    acc[1] += mi;
    acc[2] += mi * iw;
    acc[3] += mt;
    acc[4] += mt * t;
    acc[5] += mi * t;
    int q = 24;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      acc[6 + a] += mk * J[a];
      acc[12 + a] += J[a] * mi;
      acc[18 + a] += J[a] * mt;
#pragma unroll
      for (int b = a; b < 6; ++b) acc[q++] += J[a] * J[b];
    }
  }
  // warp butterflies, then warps in order
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kSums; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(LCR_FULL, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < kSums) {
    double s = 0.0;
    for (int j = 0; j < kEccThreads / 32; ++j) s += red[j][threadIdx.x];
    part[(static_cast<size_t>(f) * gridDim.x + blockIdx.x) * kSums + threadIdx.x] = s;
  }
}

// Solves the 6x6 SPD-ish system A x = b by Gaussian elimination with partial
// pivoting (FP64); returns false when singular.
__device__ bool solve6(double A[6][6], double b[6], double x[6]) {
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    for (int r = c + 1; r < 6; ++r)
      if (fabs(A[r][c]) > fabs(A[piv][c])) piv = r;
    if (!(fabs(A[piv][c]) > 0.0)) return false;
    if (piv != c) {
      for (int k = 0; k < 6; ++k) {
        const double t = A[c][k];
        A[c][k] = A[piv][k];
        A[piv][k] = t;
      }
      const double t = b[c];
      b[c] = b[piv];
      b[piv] = t;
    }
    for (int r = c + 1; r < 6; ++r) {
      const double fct = A[r][c] / A[c][c];
      for (int k = c; k < 6; ++k) A[r][k] -= fct * A[c][k];
      b[r] -= fct * b[c];
    }
  }
  for (int r = 5; r >= 0; --r) {
    double s = b[r];
    for (int k = r + 1; k < 6; ++k) s -= A[r][k] * x[k];
    x[r] = s / A[r][r];
  }
  return true;
}

// One thread per frame: sums over the blocks in order, the ECC step, the
// warp update and the convergence test |rho - rho_prev| < eps.
__global__ void k_ecc_step(const double* __restrict__ part, int nblocks, int F, float* __restrict__ warps,
                           double* __restrict__ rho, int* __restrict__ active, int* __restrict__ iters, double eps,
                           int max_iter, int* __restrict__ any_active) {
  const int f = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F || !active[f]) return;
  double s[kSums];
  for (int k = 0; k < kSums; ++k) s[k] = 0.0;
  for (int bk = 0; bk < nblocks; ++bk)
    for (int k = 0; k < kSums; ++k) s[k] += part[(static_cast<size_t>(f) * nblocks + bk) * kSums + k];
  const double n = s[0];
  iters[f] += 1;
  if (!(n > 0.0)) {
    active[f] = 0;
    return;
  }
  const double mi = s[1] / n, mt = s[3] / n;
  const double img_var = s[2] - n * mi * mi, tmp_var = s[4] - n * mt * mt;
  const double corr = s[5] - mi * s[3] - mt * s[1] + n * mi * mt;
  const double inorm = sqrt(fmax(img_var, 0.0)), tnorm = sqrt(fmax(tmp_var, 0.0));
  const double r = inorm > 0 && tnorm > 0 ? corr / (inorm * tnorm) : 0.0;
  double ip[6], tp[6], H[6][6];
  for (int a = 0; a < 6; ++a) {
    ip[a] = s[12 + a] - mi * s[6 + a];
    tp[a] = s[18 + a] - mt * s[6 + a];
  }
  int q = 24;
  for (int a = 0; a < 6; ++a)
    for (int b = a; b < 6; ++b) H[a][b] = H[b][a] = s[q++];
  // H^-1 ip and H^-1 tp
  double Hc[6][6], b1[6], hi[6], ht[6];
  for (int a = 0; a < 6; ++a) {
    for (int b = 0; b < 6; ++b) Hc[a][b] = H[a][b];
    b1[a] = ip[a];
  }
  bool ok = solve6(Hc, b1, hi);
  for (int a = 0; a < 6; ++a) {
    for (int b = 0; b < 6; ++b) Hc[a][b] = H[a][b];
    b1[a] = tp[a];
  }
  ok = ok && solve6(Hc, b1, ht);
  if (!ok) {
    active[f] = 0;
    return;
  }
  double lam_n = img_var, lam_d = corr;
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
  if (active[f]) atomicExch(any_active, 1);
}

// Frames 1.. warped onto frame 0 (inverse map), frame 0 copied.
__global__ void k_sr_warp(const float* __restrict__ in, int w, int h, const float* __restrict__ warps,
                          float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, f = blockIdx.z;
  if (x >= w) return;
  const size_t plane = static_cast<size_t>(w) * h, o = f * plane + static_cast<size_t>(y) * w + x;
  if (f == 0) {
    out[o] = in[o];
    return;
  }
  const float* m = warps + 6 * f;
  out[o] = bilinear(in + f * plane, w, h, m[0] * x + m[1] * y + m[2], m[3] * x + m[4] * y + m[5]);
}

// High-resolution ZE-mean: HR(y, x) = mean of the positive warped_k(y / s, x / s)
// (FP64 sum in frame order, divided by the count, to float; 0/0 = NaN).
__global__ void k_sr_zemean(const float* __restrict__ warped, int w, int h, int F, int s, float* __restrict__ hr) {
  const int W = w * s;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= W) return;
  const size_t src = static_cast<size_t>(y / s) * w + x / s, plane = static_cast<size_t>(w) * h;
  double sum = 0.0;
  int cnt = 0;
  for (int k = 0; k < F; ++k) {
    const float v = warped[k * plane + src];
    if (v > 0.f) {
      sum += v;
      ++cnt;
    }
  }
  hr[static_cast<size_t>(y) * W + x] = static_cast<float>(sum / cnt);
}

// Lanczos (a = 4) weights of the 8 taps at floor(p) - 3 .. floor(p) + 4 for
// the fractional position t = p - floor(p): L(d) = sinc(d) sinc(d / 4),
// normalised to sum 1; t = 0 takes the centre tap alone.
__device__ void lanczos4(float t, float wgt[8]) {
  if (t < 1.1920929e-7f) {
    for (int i = 0; i < 8; ++i) wgt[i] = i == 3 ? 1.f : 0.f;
    return;
  }
  const double pi = 3.14159265358979323846;
  double sum = 0.0, ww[8];
  for (int i = 0; i < 8; ++i) {
    const double d = (i - 3) - static_cast<double>(t);
    const double a = pi * d;
    ww[i] = 4.0 * sin(a) * sin(a / 4.0) / (a * a);
    sum += ww[i];
  }
  for (int i = 0; i < 8; ++i) wgt[i] = static_cast<float>(ww[i] / sum);
}

// Resampling by 1/s along x (pass 0) or y (pass 1): output sample o reads the
// source around p = (o + 0.5) s - 0.5, taps clamped to the image.
__global__ void k_sr_lanczos(const float* __restrict__ in, int win, int hin, int wout, int hout, int axis, int s,
                             float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= wout || y >= hout) return;
  const int o = axis == 0 ? x : y;
  const float p = (o + 0.5f) * s - 0.5f;
  const float fl = floorf(p);
  float wgt[8];
  lanczos4(p - fl, wgt);
  const int base = static_cast<int>(fl) - 3;
  float acc = 0.f;
  for (int i = 0; i < 8; ++i) {
    if (axis == 0) {
      const int xx = min(max(base + i, 0), win - 1);
      acc += wgt[i] * in[static_cast<size_t>(y) * win + xx];
    } else {
      const int yy = min(max(base + i, 0), hin - 1);
      acc += wgt[i] * in[static_cast<size_t>(yy) * win + x];
    }
  }
  out[static_cast<size_t>(y) * wout + x] = acc;
}

// uint16 by rounding half to even, saturating; NaN -> 0.
__global__ void k_sr_u16(const float* __restrict__ in, size_t n, uint16_t* __restrict__ out) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = in[i];
  float r = rintf(v);
  if (!(r > 0.f)) r = 0.f;
  if (r > 65535.f) r = 65535.f;
  out[i] = static_cast<uint16_t>(r);
}

}  // namespace

void super_resolve_run(lcr_ctx* ctx, const uint16_t* frames, int w, int h, int F, int factor, int max_iter,
                       double eps, uint16_t* out, float* warps_out, float minmax_out[2], int* iters_out) {
  const size_t plane = static_cast<size_t>(w) * h, all = plane * F;
  const int W = w * factor, H = h * factor;
  const int nblocks = std::min(64, static_cast<int>((plane + kEccThreads - 1) / kEccThreads));
  const size_t bytes = all * 2 + 6 * all * 4 + static_cast<size_t>(W) * H * 4 + static_cast<size_t>(w) * H * 4 +
                       plane * 4 + plane * 2 + F * (24 + 8 + 8) + static_cast<size_t>(F) * nblocks * kSums * 8 + 64;
  char* blk = static_cast<char*>(dev_alloc(ctx, bytes + 1024));
  char* q = blk;
  auto take = [&](size_t b) {
    char* r = q;
    q += (b + 255) & ~static_cast<size_t>(255);
    return r;
  };
  auto* d16 = reinterpret_cast<uint16_t*>(take(all * 2));
  auto* img = reinterpret_cast<float*>(take(all * 4));
  auto* tmp = reinterpret_cast<float*>(take(all * 4));
  auto* blur = reinterpret_cast<float*>(take(all * 4));
  auto* gx = reinterpret_cast<float*>(take(all * 4));
  auto* gy = reinterpret_cast<float*>(take(all * 4));
  auto* warped = reinterpret_cast<float*>(take(all * 4));
  auto* hr = reinterpret_cast<float*>(take(static_cast<size_t>(W) * H * 4));
  auto* half = reinterpret_cast<float*>(take(static_cast<size_t>(w) * H * 4));
  auto* lr = reinterpret_cast<float*>(take(plane * 4));
  auto* o16 = reinterpret_cast<uint16_t*>(take(plane * 2));
  auto* warps = reinterpret_cast<float*>(take(F * 24));
  auto* rho = reinterpret_cast<double*>(take(F * 8));
  auto* active = reinterpret_cast<int*>(take(F * 4));
  auto* iters = reinterpret_cast<int*>(take(F * 4));
  auto* part = reinterpret_cast<double*>(take(static_cast<size_t>(F) * nblocks * kSums * 8));
  auto* flags = reinterpret_cast<unsigned int*>(take(64));
  CUDA_TRY(cudaMemcpyAsync(d16, frames, all * 2, cudaMemcpyHostToDevice, ctx->stream));
  const unsigned int init[3] = {0xffffffffu, 0u, 0u};
  CUDA_TRY(cudaMemcpyAsync(flags, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
  LCR_LAUNCH(ctx, k_sr_float, static_cast<unsigned>((all + 255) / 256), 256, 0, d16, all, img, flags);
  // 5x5 Gaussian, sigma 0.3 ((5 - 1) / 2 - 1) + 0.8 = 1.1
  const double sg = 1.1;
  double g[3] = {1.0, std::exp(-1.0 / (2 * sg * sg)), std::exp(-4.0 / (2 * sg * sg))};
  const double gs = g[0] + 2 * g[1] + 2 * g[2];
  const float g0 = static_cast<float>(g[0] / gs), g1 = static_cast<float>(g[1] / gs), g2 = static_cast<float>(g[2] / gs);
  const dim3 gimg((w + 127) / 128, h, F);
  LCR_LAUNCH(ctx, k_sr_blur_h, gimg, 128, 0, img, w, h, g0, g1, g2, tmp);
  LCR_LAUNCH(ctx, k_sr_blur_v, gimg, 128, 0, tmp, w, h, g0, g1, g2, blur);
  LCR_LAUNCH(ctx, k_sr_grad, gimg, 128, 0, blur, w, h, gx, gy);
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
  for (int it = 0; it < max_iter && F > 1; ++it) {
    CUDA_TRY(cudaMemsetAsync(flags + 2, 0, 4, ctx->stream));
    LCR_LAUNCH(ctx, k_ecc_pass, dim3(nblocks, F - 1), kEccThreads, 0, blur, blur, gx, gy, w, h, warps, active, part);
    LCR_LAUNCH(ctx, k_ecc_step, (F + 63) / 64, 64, 0, part, nblocks, F, warps, rho, active, iters, eps, max_iter,
               reinterpret_cast<int*>(flags + 2));
    int any = 0;
    CUDA_TRY(cudaMemcpyAsync(&any, flags + 2, 4, cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
    if (!any) break;
  }
  LCR_LAUNCH(ctx, k_sr_warp, gimg, 128, 0, img, w, h, warps, warped);
  LCR_LAUNCH(ctx, k_sr_zemean, dim3((W + 127) / 128, H), 128, 0, warped, w, h, F, factor, hr);
  LCR_LAUNCH(ctx, k_sr_lanczos, dim3((w + 127) / 128, H), 128, 0, hr, W, H, w, H, 0, factor, half);
  LCR_LAUNCH(ctx, k_sr_lanczos, dim3((w + 127) / 128, h), 128, 0, half, w, H, w, h, 1, factor, lr);
  LCR_LAUNCH(ctx, k_sr_u16, static_cast<unsigned>((plane + 255) / 256), 256, 0, lr, plane, o16);
  CUDA_TRY(cudaMemcpyAsync(out, o16, plane * 2, cudaMemcpyDeviceToHost, ctx->stream));
  if (warps_out) CUDA_TRY(cudaMemcpyAsync(warps_out, warps, F * 24, cudaMemcpyDeviceToHost, ctx->stream));
  if (iters_out) CUDA_TRY(cudaMemcpyAsync(iters_out, iters, F * 4, cudaMemcpyDeviceToHost, ctx->stream));
  unsigned int mm[2];
  CUDA_TRY(cudaMemcpyAsync(mm, flags, 8, cudaMemcpyDeviceToHost, ctx->stream));
  sync(ctx);
  if (minmax_out) {
    minmax_out[0] = mm[1] ? static_cast<float>(mm[0]) : 0.f;
    minmax_out[1] = static_cast<float>(mm[1]);
  }
  dev_free(ctx, blk);
}
