// CPU restatement of the super-resolution front end -- TEST INFRASTRUCTURE
// ONLY (the CPU baseline of bench.py's super-resolution workload, and a second
// check of oracle/sr.py).  Nothing in the shipped library links or calls it.
//
// It follows capture/super_resolution/super_resolution.cpp:236-314 with the
// published methods oracle/sr.py restates (OpenCV, which the reference calls,
// is absent; parity unpinned): a 5x5 Gaussian of sigma 1.1 with reflect-101
// borders, central-difference gradients, ECC affine registration
// (Evangelidis & Psarakis 2008) over the pixels whose four bilinear taps lie
// inside the frame, with every sum in FP64 and the Gauss-Newton step by LU
// with partial pivoting; stop when the correlation coefficient changes by
// less than eps; the inverse-map bilinear warp (zero border), the
// zero-eliminated mean (FP64 sum in frame order), nearest upsampling and
// separable Lanczos-4 resampling (taps clamped), rounding half to even.  The
// frames register in parallel (OpenMP), as the reference's loop at :256 does.
//
// Sums run in a different order from numpy's, so results agree with
// oracle/sr.py to rounding, not bit for bit.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

int reflect101(int i, int n) {
  if (n == 1) return 0;
  while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
  return i;
}

// Separable 5-tap smoothing, horizontal then vertical, in FP32.
void gauss5(const float* in, int w, int h, float* out) {
  const double s = 1.1;
  const double g64[3] = {1.0, std::exp(-1.0 / (2 * s * s)), std::exp(-4.0 / (2 * s * s))};
  const double gs = g64[0] + 2 * g64[1] + 2 * g64[2];
  const float g[3] = {static_cast<float>(g64[0] / gs), static_cast<float>(g64[1] / gs),
                      static_cast<float>(g64[2] / gs)};
  std::vector<float> tmp(static_cast<size_t>(w) * h);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const float* r = in + static_cast<size_t>(y) * w;
      auto at = [&](int o) { return r[reflect101(x + o, w)]; };
      const float a = g[0] * at(0), b = g[1] * (at(-1) + at(1)), c = g[2] * (at(-2) + at(2));
      tmp[static_cast<size_t>(y) * w + x] = (a + b) + c;
    }
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      auto at = [&](int o) { return tmp[static_cast<size_t>(reflect101(y + o, h)) * w + x]; };
      const float a = g[0] * at(0), b = g[1] * (at(-1) + at(1)), c = g[2] * (at(-2) + at(2));
      out[static_cast<size_t>(y) * w + x] = (a + b) + c;
    }
}

void grad(const float* f, int w, int h, float* gx, float* gy) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t o = static_cast<size_t>(y) * w + x;
      gx[o] = 0.5f * (f[static_cast<size_t>(y) * w + reflect101(x + 1, w)] -
                      f[static_cast<size_t>(y) * w + reflect101(x - 1, w)]);
      gy[o] = 0.5f * (f[static_cast<size_t>(reflect101(y + 1, h)) * w + x] -
                      f[static_cast<size_t>(reflect101(y - 1, h)) * w + x]);
    }
}

// Bilinear sample with a zero border (a tap outside contributes 0).
float bilinear(const float* f, int w, int h, float u, float v) {
  const float fu = std::floor(u), fv = std::floor(v);
  const long x0 = static_cast<long>(fu), y0 = static_cast<long>(fv);
  const float ax = u - fu, ay = v - fv;
  auto at = [&](long xx, long yy) {
    return (xx >= 0 && yy >= 0 && xx < w && yy < h) ? f[static_cast<size_t>(yy) * w + xx] : 0.f;
  };
  const float top = at(x0, y0) * (1.f - ax) + at(x0 + 1, y0) * ax;
  const float bot = at(x0, y0 + 1) * (1.f - ax) + at(x0 + 1, y0 + 1) * ax;
  return top * (1.f - ay) + bot * ay;
}

// Solves A x = b (6x6) by Gaussian elimination with partial pivoting; false
// when singular.
bool solve6(double A[6][6], double b[6], double x[6]) {
  for (int c = 0; c < 6; ++c) {
    int piv = c;
    for (int r = c + 1; r < 6; ++r)
      if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
    if (!(std::fabs(A[piv][c]) > 0.0)) return false;
    if (piv != c) {
      for (int k = 0; k < 6; ++k) std::swap(A[c][k], A[piv][k]);
      std::swap(b[c], b[piv]);
    }
    for (int r = c + 1; r < 6; ++r) {
      const double f = A[r][c] / A[c][c];
      for (int k = c; k < 6; ++k) A[r][k] -= f * A[c][k];
      b[r] -= f * b[c];
    }
  }
  for (int r = 5; r >= 0; --r) {
    double s = b[r];
    for (int k = r + 1; k < 6; ++k) s -= A[r][k] * x[k];
    x[r] = s / A[r][r];
  }
  return true;
}

// Whether H (symmetric) is positive definite: a Cholesky factorisation runs.
bool positive_definite(const double H[6][6]) {
  double L[6][6] = {};
  for (int j = 0; j < 6; ++j) {
    double d = H[j][j];
    for (int k = 0; k < j; ++k) d -= L[j][k] * L[j][k];
    if (!(d > 0.0)) return false;
    L[j][j] = std::sqrt(d);
    for (int i = j + 1; i < 6; ++i) {
      double t = H[i][j];
      for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
      L[i][j] = t / L[j][j];
    }
  }
  return true;
}

// ECC affine registration of img (with gradients gx, gy) to tmpl; m is the
// 2x3 inverse map (row-major), starting at the identity.  Returns iterations.
int ecc_affine(const float* tmpl, const float* img, const float* gx, const float* gy, int w, int h, int iters,
               double eps, float m[6]) {
  const size_t n = static_cast<size_t>(w) * h;
  std::vector<float> I(n), GX(n), GY(n);
  std::vector<uint8_t> mk(n);
  double prev = -1.0;
  int it = 0;
  for (it = 1; it <= iters; ++it) {
    double cnt = 0, si = 0, st = 0;
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t o = static_cast<size_t>(y) * w + x;
        const float u = m[0] * x + m[1] * y + m[2], v = m[3] * x + m[4] * y + m[5];
        I[o] = bilinear(img, w, h, u, v);
        GX[o] = bilinear(gx, w, h, u, v);
        GY[o] = bilinear(gy, w, h, u, v);
        const float fu = std::floor(u), fv = std::floor(v);
        mk[o] = fu >= 0.f && fv >= 0.f && fu + 1.f < w && fv + 1.f < h;
        if (mk[o]) {
          cnt += 1;
          si += I[o];
          st += tmpl[o];
        }
      }
    if (!(cnt > 0)) break;
    const double mi = si / cnt, mt = st / cnt;
    double H[6][6] = {}, ip[6] = {}, tp[6] = {}, corr = 0, ii = 0, tt = 0;
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t o = static_cast<size_t>(y) * w + x;
        if (!mk[o]) continue;
        const double X = x, Y = y, g1 = GX[o], g2 = GY[o];
        const double J[6] = {X * g1, X * g2, Y * g1, Y * g2, g1, g2};
        const double iz = I[o] - mi, tz = tmpl[o] - mt;
        corr += iz * tz;
        ii += iz * iz;
        tt += tz * tz;
        for (int a = 0; a < 6; ++a) {
          ip[a] += J[a] * iz;
          tp[a] += J[a] * tz;
          for (int b = a; b < 6; ++b) H[a][b] += J[a] * J[b];
        }
      }
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < a; ++b) H[a][b] = H[b][a];
    const double r = ii > 0 && tt > 0 ? corr / (std::sqrt(ii) * std::sqrt(tt)) : 0.0;
    if (!positive_definite(H)) break;
    double A[6][6], bb[6], hi[6], ht[6];
    std::memcpy(A, H, sizeof A);
    std::memcpy(bb, ip, sizeof bb);
    if (!solve6(A, bb, hi)) break;
    std::memcpy(A, H, sizeof A);
    std::memcpy(bb, tp, sizeof bb);
    if (!solve6(A, bb, ht)) break;
    double lam_n = ii, lam_d = corr;
    for (int a = 0; a < 6; ++a) {
      lam_n -= ip[a] * hi[a];
      lam_d -= tp[a] * hi[a];
    }
    if (!(lam_d > 0)) break;
    const double lam = lam_n / lam_d;
    double dp[6];
    for (int a = 0; a < 6; ++a) dp[a] = lam * ht[a] - hi[a];
    m[0] += static_cast<float>(dp[0]);
    m[3] += static_cast<float>(dp[1]);
    m[1] += static_cast<float>(dp[2]);
    m[4] += static_cast<float>(dp[3]);
    m[2] += static_cast<float>(dp[4]);
    m[5] += static_cast<float>(dp[5]);
    if (std::fabs(r - prev) < eps) break;
    prev = r;
  }
  return it > iters ? iters : it;
}

// Lanczos-4 taps of output o of a resampling by 1/s (see k_sr_lanczos_h).
void lanczos4(double t, float w8[8]) {
  if (t < 1.1920929e-7) {
    for (int i = 0; i < 8; ++i) w8[i] = i == 3 ? 1.f : 0.f;
    return;
  }
  const double pi = 3.14159265358979323846;
  double ww[8], sum = 0;
  for (int i = 0; i < 8; ++i) {
    const double a = pi * ((i - 3) - t);
    ww[i] = 4 * std::sin(a) * std::sin(a / 4) / (a * a);
    sum += ww[i];
  }
  for (int i = 0; i < 8; ++i) w8[i] = static_cast<float>(ww[i] / sum);
}

}  // namespace

extern "C" {

void orc_super_resolve(const void* frames, int f32, int F, int w, int h, int factor, int iters, double eps,
                       void* out, float* warps, int* iterations) {
  const size_t plane = static_cast<size_t>(w) * h;
  std::vector<float> img(plane * F), blur(plane * F), gx(plane * F), gy(plane * F);
  for (size_t i = 0; i < plane * F; ++i)
    img[i] = f32 ? static_cast<const float*>(frames)[i] : static_cast<const uint16_t*>(frames)[i];
#pragma omp parallel for schedule(dynamic)
  for (int f = 0; f < F; ++f) {
    gauss5(&img[plane * f], w, h, &blur[plane * f]);
    grad(&blur[plane * f], w, h, &gx[plane * f], &gy[plane * f]);
  }
  for (int f = 0; f < F; ++f) {
    const float id[6] = {1, 0, 0, 0, 1, 0};
    std::memcpy(warps + 6 * f, id, sizeof id);
    iterations[f] = 0;
  }
#pragma omp parallel for schedule(dynamic)
  for (int f = 1; f < F; ++f)
    iterations[f] = ecc_affine(&blur[0], &blur[plane * f], &gx[plane * f], &gy[plane * f], w, h, iters, eps,
                               warps + 6 * f);
  // warp + zero-eliminated mean on the sensor grid (nearest upsampling commutes with it)
  std::vector<float> ze(plane);
#pragma omp parallel for
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t o = static_cast<size_t>(y) * w + x;
      double sum = 0;
      int cnt = 0;
      for (int f = 0; f < F; ++f) {
        const float* m = warps + 6 * f;
        const float v = f == 0 ? img[o]
                               : bilinear(&img[plane * f], w, h, m[0] * x + m[1] * y + m[2], m[3] * x + m[4] * y + m[5]);
        if (v > 0.f) {
          sum += v;
          ++cnt;
        }
      }
      ze[o] = cnt == 0 && f32 ? 0.f : static_cast<float>(sum / cnt);
    }
  // Lanczos-4 downsampling of the upsampled image: rows, then columns
  const int W = w * factor, H = h * factor;
  std::vector<int> xb(w), yb(h);
  std::vector<float> xw(8 * w), yw(8 * h);
  for (int o = 0; o < w; ++o) {
    const double p = (o + 0.5) * factor - 0.5, fl = std::floor(p);
    xb[o] = static_cast<int>(fl) - 3;
    lanczos4(static_cast<float>(p - fl), &xw[8 * o]);
  }
  for (int o = 0; o < h; ++o) {
    const double p = (o + 0.5) * factor - 0.5, fl = std::floor(p);
    yb[o] = static_cast<int>(fl) - 3;
    lanczos4(static_cast<float>(p - fl), &yw[8 * o]);
  }
  std::vector<float> half(plane);
#pragma omp parallel for
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float acc = 0.f;
      for (int i = 0; i < 8; ++i) {
        const int xx = std::min(std::max(xb[x] + i, 0), W - 1) / factor;
        acc += xw[8 * x + i] * ze[static_cast<size_t>(y) * w + xx];
      }
      half[static_cast<size_t>(y) * w + x] = acc;
    }
#pragma omp parallel for
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float acc = 0.f;
      for (int i = 0; i < 8; ++i) {
        const int yy = std::min(std::max(yb[y] + i, 0), H - 1) / factor;
        acc += yw[8 * y + i] * half[static_cast<size_t>(yy) * w + x];
      }
      const size_t o = static_cast<size_t>(y) * w + x;
      if (f32) {
        static_cast<float*>(out)[o] = acc;
      } else {
        float r = std::nearbyint(acc);
        if (!(r > 0.f)) r = 0.f;
        if (r > 65535.f) r = 65535.f;
        static_cast<uint16_t*>(out)[o] = static_cast<uint16_t>(r);
      }
    }
}

}  // extern "C"
