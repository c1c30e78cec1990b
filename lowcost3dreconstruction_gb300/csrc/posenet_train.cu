// Pose proposal: pair head (forward and backward), loss, encoder backward,
// AdamW, and the conversions between the network's output and 4x4 poses.
//
// The head's forward layers are tcgen05 GEMMs (k_gemm_tc).  The backward
// pass runs on the CUDA cores with one thread per output and a fixed
// summation order, so gradients are bit-reproducible run to run.  The
// encoder's max-pool makes its backward sparse: a pooled channel's gradient
// flows only into the point that won the max, so dW3 is a gather over the
// (cloud, channel) arg-max rows of the stored layer-2 activations, and the
// layers below see only the points that won at least one channel.
#include <cuda_bf16.h>

#include <cmath>

#include "posenet.cuh"
#include "tc.cuh"

using bf16 = __nv_bfloat16;

namespace {

using namespace posenet;

__device__ __forceinline__ float ld(const float* p) { return *p; }
__device__ __forceinline__ float ld(const bf16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ------------------------------------------------------------------ GEMM
// C(m, n) = sum_k A(m, k) B(n, k), A(m, k) = A[m*sam + k*sak], B(n, k) =
// B[n*sbn + k*sbk]; 64x64 tiles, 4x4 outputs per thread, each output summed
// over k in ascending order.  Epilogue: + bias[n], ReLU, x (mask(m, n) > 0),
// then f32 and/or bf16 stores with row stride ldo.
struct Epi {
  const float* bias = nullptr;
  bool relu = false;
  const bf16* mask = nullptr;
  long long ldm = 0;
  float* out = nullptr;
  bf16* outb = nullptr;
  long long ldo = 0;
};

template <typename TA, typename TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const TA* __restrict__ A, long long sam,
                                              long long sak, const TB* __restrict__ Bm, long long sbn, long long sbk,
                                              Epi e) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int t = 0; t < 4; ++t) {
      const int idx = tid + 256 * t;
      // k fastest when k is the contiguous index, else the row index fastest
      const int ra = sak == 1 ? idx >> 4 : idx & 63, ca = sak == 1 ? idx & 15 : idx >> 6;
      const int m = m0 + ra, k = k0 + ca;
      As[ca][ra] = (m < M && k < K) ? ld(A + m * sam + k * sak) : 0.f;
      const int rb = sbk == 1 ? idx >> 4 : idx & 63, cb = sbk == 1 ? idx & 15 : idx >> 6;
      const int n = n0 + rb, kb = k0 + cb;
      Bs[cb][rb] = (n < N && kb < K) ? ld(Bm + n * sbn + kb * sbk) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= N) continue;
      float v = acc[i][j];
      if (e.bias) v += e.bias[n];
      if (e.relu) v = fmaxf(v, 0.f);
      if (e.mask && !(__bfloat162float(e.mask[m * e.ldm + n]) > 0.f)) v = 0.f;
      if (e.out) e.out[m * e.ldo + n] = v;
      if (e.outb) e.outb[m * e.ldo + n] = __float2bfloat16_rn(v);
    }
  }
}

template <typename TA, typename TB>
void gemm(lcr_ctx* ctx, int M, int N, int K, const TA* A, long long sam, long long sak, const TB* B, long long sbn,
          long long sbk, const Epi& e) {
  if (M == 0 || N == 0) return;
  const dim3 grid((N + 63) / 64, (M + 63) / 64);
  LCR_LAUNCH(ctx, (k_gemm<TA, TB>), grid, 256, 0, M, N, K, A, sam, sak, B, sbn, sbk, e);
}

// ------------------------------------------------------ tensor-core GEMM
// C[m][n] = act(sum_k A[m][k] B[n][k] + bias[n]) with A [M][K] and B [N][K]
// bf16 row-major (both K-major), fp32 accumulation in TMEM: the head's
// forward layers.  One CTA (4 warps) per 128-row tile of A and NT-column tile
// of B.  K runs in 64-wide steps through two shared-memory stages: the threads
// copy one step's tiles into the 128-byte swizzled layout while the tensor
// core multiplies the previous step's (one elected thread issues four
// 128 x NT x 16 MMAs per step).  Thread t then reads TMEM lane t (row m0 + t)
// for the epilogue.  Rows past M and columns past N are zero-filled on load
// and skipped on store.  K must be a multiple of 64.  Every wait is bounded;
// a timeout drains the MMAs issued and raises *err.
template <int NT>
__global__ void __launch_bounds__(128) k_gemm_tc(int M, int N, int K, const bf16* __restrict__ A,
                                                 const bf16* __restrict__ Bm, Epi e, int* __restrict__ err) {
  constexpr int kATile = 128 * 128;  // 128 rows x 64 bf16
  constexpr int kBTile = NT * 128;
  constexpr int kStage = kATile + kBTile;
  constexpr int kCols = NT < 32 ? 32 : NT;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * kStage);  // [0..1] stage MMAs done, [2] drain
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 3);
  volatile int* flag = reinterpret_cast<volatile int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * NT;
  if (tid == 0) {
    for (int i = 0; i < 3; ++i) tc::mbar_init(&bar[i], 1);
    *flag = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc<kCols>(tslot);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  auto load = [&](int ks, int st) {
    unsigned char* a = sm + st * kStage;
    unsigned char* b = a + kATile;
    const int k0 = ks * 64;
    for (int i = tid; i < 128 * 8; i += 128) {
      const int r = i >> 3, c = i & 7;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (m0 + r < M) v = *reinterpret_cast<const uint4*>(A + static_cast<size_t>(m0 + r) * K + k0 + c * 8);
      *reinterpret_cast<uint4*>(a + r * 128 + ((c ^ (r & 7)) << 4)) = v;
    }
    for (int i = tid; i < NT * 8; i += 128) {
      const int r = i >> 3, c = i & 7;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (n0 + r < N) v = *reinterpret_cast<const uint4*>(Bm + static_cast<size_t>(n0 + r) * K + k0 + c * 8);
      *reinterpret_cast<uint4*>(b + r * 128 + ((c ^ (r & 7)) << 4)) = v;
    }
    tc::fence_async_smem();
  };
  const uint32_t idesc = tc::idesc_bf16_f32(128, NT);
  const int nk = K / 64;
  uint32_t ph[2] = {0u, 0u};
  load(0, 0);
  for (int ks = 0; ks < nk; ++ks) {
    const int st = ks & 1;
    __syncthreads();  // the stage is written by every thread
    if (*flag) break;
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t a = tc::smem_u32(sm + st * kStage), b = a + kATile;
      for (int s = 0; s < 4; ++s)
        tc::mma_bf16(tmem, tc::sdesc_sw128(a + s * 32), tc::sdesc_sw128(b + s * 32), idesc, ks > 0 || s > 0);
      tc::mma_commit(&bar[st]);
    }
    if (ks + 1 < nk) {
      // the other stage was read by step ks-1's MMAs
      if (ks >= 1) {
        if (!tc::mbar_wait(&bar[st ^ 1], ph[st ^ 1])) *flag = 1;
        ph[st ^ 1] ^= 1;
      }
      load(ks + 1, st ^ 1);
    }
  }
  __syncthreads();
  if (tid == 0) tc::mma_commit(&bar[2]);  // behind every MMA issued
  if (!tc::mbar_wait(&bar[2], 0)) *flag = 1;
  tc::tc_fence_after();
  const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
  const int m = m0 + tid;
  for (int c0 = 0; c0 < NT; c0 += 32) {
    float v[32];
    tc::tmem_ld32(tmem + lane_base + c0, v);
    if (m >= M || *flag) continue;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int n = n0 + c0 + j;
      if (c0 + j >= NT || n >= N) break;
      float x = v[j];
      if (e.bias) x += e.bias[n];
      if (e.relu) x = fmaxf(x, 0.f);
      if (e.out) e.out[m * e.ldo + n] = x;
      if (e.outb) e.outb[m * e.ldo + n] = __float2bfloat16_rn(x);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_free<kCols>(tmem);
  }
  if (*flag && tid == 0) atomicExch(err, 1);
}

template <int NT>
void gemm_tc(lcr_ctx* ctx, int M, int N, int K, const bf16* A, const bf16* B, const Epi& e, int* err) {
  if (M == 0 || N == 0) return;
  if (K % 64 != 0) LCR_THROW(LCR_ERR_INVALID_ARG, "tensor-core GEMM needs K a multiple of 64 (K=%d)", K);
  const int smem = 2 * (128 * 128 + NT * 128) + 64 + 1024;
  CUDA_TRY(cudaFuncSetAttribute(k_gemm_tc<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const dim3 grid((N + NT - 1) / NT, (M + 127) / 128);
  LCR_LAUNCH(ctx, k_gemm_tc<NT>, grid, 128, smem, M, N, K, A, B, e, err);
}

// out[c] = sum over rows of src[r][c], rows in order.
__global__ void k_colsum(const float* __restrict__ src, int rows, int cols, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += src[static_cast<size_t>(r) * cols + c];
  out[c] = s;
}

// ------------------------------------------------------------------ loss
// L = (1/B) sum_b sum_i (y - label)^2 over the 9 outputs (r6 and the scaled
// residual translation); dy = 2 (y - label) / B.  One block, fixed order.
__global__ void __launch_bounds__(256) k_loss(const float* __restrict__ y, const float* __restrict__ lab, int B,
                                              float* __restrict__ dy, float* __restrict__ loss) {
  __shared__ float red[256];
  float acc = 0.f;
  for (int b = threadIdx.x; b < B; b += 256) {
    float l = 0.f;
    for (int i = 0; i < kOut; ++i) {
      const float d = y[b * kOut + i] - lab[b * kOut + i];
      l += d * d;
      dy[b * kOut + i] = 2.0f * d / static_cast<float>(B);
    }
    acc += l;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0] / static_cast<float>(B);
}

// ------------------------------------------------------- encoder backward
// Gradient reaching a pooled channel: d feature, zero where the ReLU after
// the max was inactive.
__device__ __forceinline__ float pooled_grad(const float* feat, const float* dx0, int B, int cl, int c) {
  if (!(feat[static_cast<size_t>(cl) * kF3 + c] > 0.f)) return 0.f;
  const int row = cl < B ? cl : cl - B, col = (cl < B ? 0 : kF3) + c;
  return dx0[static_cast<size_t>(row) * kIn + col];
}

// dW3[c][k] = sum_clouds dm(cl, c) h2(cl, argmax(cl, c), k), db3[c] = sum dm.
// One warp per channel, 4 k per lane, clouds in order.
__global__ void __launch_bounds__(256) k_bwd_w3(const float* __restrict__ feat, const float* __restrict__ dx0,
                                                const int* __restrict__ argmax, const bf16* __restrict__ h2g, int B,
                                                float* __restrict__ grad) {
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= kF3) return;
  float acc[4] = {0.f, 0.f, 0.f, 0.f}, db = 0.f;
  for (int cl = 0; cl < 2 * B; ++cl) {
    const float dm = pooled_grad(feat, dx0, B, cl, c);
    if (dm == 0.f) continue;
    const int p = argmax[static_cast<size_t>(cl) * kF3 + c];
    const uint2 raw = *reinterpret_cast<const uint2*>(h2g + (static_cast<size_t>(cl) * kPts + p) * kF2 + lane * 4);
    const bf16* h = reinterpret_cast<const bf16*>(&raw);
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = fmaf(dm, __bfloat162float(h[j]), acc[j]);
    db += dm;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) grad[oW3 + static_cast<size_t>(c) * kF2 + lane * 4 + j] = acc[j];
  if (lane == 0) grad[oB3 + c] = db;
}

// Per-cloud gradient partials of W1, b1, W2, b2 (layout of the parameter
// vector from oW1 on).  Channels with a nonzero pooled gradient are sorted by
// (arg-max point, channel); each point that won channels gets
//   dh2 = sum over its channels of dm(c) W3[c]   (channel order),
//   dz2 = dh2 (h2 > 0), dh1 = W2^T dz2, dz1 = dh1 (h1 > 0),
// and the points are processed in ascending order, 32 at a time.
constexpr int kSlots = 32;
constexpr int kSegCap = kF3 + 4;  // segment starts (<= 1025), padded to keep what follows 16-byte aligned
constexpr size_t kBwdSmem = 4 * (kF3 + kF3 + kSegCap + kF2 * kF1 + 4 * kF1 + kSlots * (kF2 + kF1 + kF1 + 4));

__global__ void __launch_bounds__(256) k_bwd_cloud(const float4* __restrict__ pts, const float* __restrict__ feat,
                                                   const float* __restrict__ dx0, const int* __restrict__ argmax,
                                                   const bf16* __restrict__ h2g, const float* __restrict__ w,
                                                   const bf16* __restrict__ w2b, const bf16* __restrict__ w3b, int B,
                                                   float* __restrict__ part) {
  extern __shared__ float sm[];
  uint32_t* keys = reinterpret_cast<uint32_t*>(sm);          // [1024]
  float* dm = sm + kF3;                                       // [1024]
  int* seg = reinterpret_cast<int*>(sm + 2 * kF3);            // [kSegCap]
  float* w2f = sm + 2 * kF3 + kSegCap;                        // [128][64]
  float4* w1s = reinterpret_cast<float4*>(w2f + kF2 * kF1);   // [64]  (w0, w1, w2, b1)
  float* dz2s = reinterpret_cast<float*>(w1s + kF1);          // [32][128]
  float* h1s = dz2s + kSlots * kF2;                           // [32][64]
  float* dz1s = h1s + kSlots * kF1;                           // [32][64]
  float4* xs = reinterpret_cast<float4*>(dz1s + kSlots * kF1);  // [32]
  __shared__ int nseg_s, nvalid_s;

  const int cl = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int c = tid; c < kF3; c += 256) {
    const float d = pooled_grad(feat, dx0, B, cl, c);
    dm[c] = d;
    keys[c] = d != 0.f ? (static_cast<uint32_t>(argmax[static_cast<size_t>(cl) * kF3 + c]) << 10) | c : 0xffffffffu;
  }
  for (int i = tid; i < kF2 * kF1; i += 256) w2f[i] = __bfloat162float(w2b[i]);
  for (int i = tid; i < kF1; i += 256)
    w1s[i] = make_float4(bf16r(w[oW1 + 3 * i]), bf16r(w[oW1 + 3 * i + 1]), bf16r(w[oW1 + 3 * i + 2]), w[oB1 + i]);
  __syncthreads();
  // bitonic sort of the 1024 keys
  for (int k = 2; k <= kF3; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < kF3; i += 256) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint32_t a = keys[i], b = keys[ixj];
          if ((a > b) == ((i & k) == 0)) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  // segment starts (one per point that won a channel), by warp 0
  if (warp == 0) {
    int cnt = 0;
    const int i0 = lane * 32;
    for (int i = i0; i < i0 + 32; ++i)
      if (keys[i] != 0xffffffffu && (i == 0 || (keys[i] >> 10) != (keys[i - 1] >> 10))) ++cnt;
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(LCR_FULL, incl, o);
      if (lane >= o) incl += t;
    }
    int pos = incl - cnt;
    for (int i = i0; i < i0 + 32; ++i)
      if (keys[i] != 0xffffffffu && (i == 0 || (keys[i] >> 10) != (keys[i - 1] >> 10))) seg[pos++] = i;
    int nv = 0;
    for (int i = i0; i < i0 + 32; ++i) nv += keys[i] != 0xffffffffu;
    for (int o = 16; o > 0; o >>= 1) nv += __shfl_xor_sync(LCR_FULL, nv, o);
    if (lane == 31) nseg_s = incl;
    if (lane == 0) nvalid_s = nv;
  }
  __syncthreads();
  const int nseg = nseg_s;
  if (tid == 0) seg[nseg] = nvalid_s;
  __syncthreads();

  float accw2[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) accw2[i] = 0.f;
  float accb2 = 0.f, accw1 = 0.f;
  const int f2 = tid >> 1, k2 = (tid & 1) * 32;
  for (int base = 0; base < nseg; base += kSlots) {
    const int ns = min(kSlots, nseg - base);
    for (int s = warp; s < ns; s += 8) {
      const int st = seg[base + s], en = seg[base + s + 1];
      const int p = static_cast<int>(keys[st] >> 10);
      float dh[4] = {0.f, 0.f, 0.f, 0.f};
      for (int i = st; i < en; ++i) {
        const int c = static_cast<int>(keys[i] & 1023u);
        const float d = dm[c];
#pragma unroll
        for (int j = 0; j < 4; ++j) dh[j] = fmaf(d, __bfloat162float(w3b[c * kF2 + lane + 32 * j]), dh[j]);
      }
      const bf16* h2 = h2g + (static_cast<size_t>(cl) * kPts + p) * kF2;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        dz2s[s * kF2 + lane + 32 * j] = __bfloat162float(h2[lane + 32 * j]) > 0.f ? dh[j] : 0.f;
      const float4 x = pts[static_cast<size_t>(cl) * kPts + p];
      if (lane == 0) xs[s] = x;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float4 wv = w1s[lane + 32 * j];
        float a = wv.w;
        a = fmaf(wv.x, x.x, a);
        a = fmaf(wv.y, x.y, a);
        a = fmaf(wv.z, x.z, a);
        h1s[s * kF1 + lane + 32 * j] = bf16r(fmaxf(a, 0.f));
      }
    }
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
      const float d = dz2s[s * kF2 + f2];
#pragma unroll
      for (int i = 0; i < 32; ++i) accw2[i] = fmaf(d, h1s[s * kF1 + k2 + i], accw2[i]);
    }
    if (tid < kF2)
      for (int s = 0; s < ns; ++s) accb2 += dz2s[s * kF2 + tid];
    // dz1 for (slot, 8 features) per thread
    {
      const int s = tid >> 3, kk = (tid & 7) * 8;
      if (s < ns) {
        float d1[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int f = 0; f < kF2; ++f) {
          const float g = dz2s[s * kF2 + f];
#pragma unroll
          for (int i = 0; i < 8; ++i) d1[i] = fmaf(g, w2f[f * kF1 + kk + i], d1[i]);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) dz1s[s * kF1 + kk + i] = h1s[s * kF1 + kk + i] > 0.f ? d1[i] : 0.f;
      }
    }
    __syncthreads();
    if (tid < 3 * kF1) {
      const int j = tid / 3, i = tid % 3;
      for (int s = 0; s < ns; ++s) {
        const float4 x = xs[s];
        accw1 = fmaf(dz1s[s * kF1 + j], i == 0 ? x.x : (i == 1 ? x.y : x.z), accw1);
      }
    } else {
      const int j = tid - 3 * kF1;
      for (int s = 0; s < ns; ++s) accw1 += dz1s[s * kF1 + j];
    }
    __syncthreads();
  }
  float* out = part + static_cast<size_t>(cl) * kEncLow;
  if (tid < 3 * kF1) out[oW1 + tid] = accw1;
  else out[oB1 + (tid - 3 * kF1)] = accw1;
#pragma unroll
  for (int i = 0; i < 32; ++i) out[oW2 + f2 * kF1 + k2 + i] = accw2[i];
  if (tid < kF2) out[oB2 + tid] = accb2;
}

// grad[oW1 + j] = sum over clouds of part[cl][j], clouds in order.
__global__ void k_reduce_part(const float* __restrict__ part, int clouds, float* __restrict__ grad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= kEncLow) return;
  float s = 0.f;
  for (int c = 0; c < clouds; ++c) s += part[static_cast<size_t>(c) * kEncLow + j];
  grad[oW1 + j] = s;
}

// ----------------------------------------------------------------- AdamW
__global__ void k_adamw(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, float lr, float b1, float b2, float eps, float wd, float bc1,
                        float bc2) {
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < kParams;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * ((mi / bc1) / (sqrtf(vi / bc2) + eps) + wd * w[i]);
  }
}

// ------------------------------------------------------------------ poses
// Network output -> row-major 4x4 source-to-target guess:
// R from the two predicted columns (Gram-Schmidt, FP64), t = c_tgt + delta/kScale - R c_src.
__global__ void k_poses(const float* __restrict__ y, const double* __restrict__ cen, int B, float* __restrict__ T) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float* o = y + b * kOut;
  double a1[3] = {o[0], o[1], o[2]}, a2[3] = {o[3], o[4], o[5]};
  double n1 = sqrt(a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2]);
  double c0[3] = {1, 0, 0}, c1[3] = {0, 1, 0}, c2[3];
  if (n1 > 1e-12) {
    for (int i = 0; i < 3; ++i) c0[i] = a1[i] / n1;
    const double d = c0[0] * a2[0] + c0[1] * a2[1] + c0[2] * a2[2];
    double u[3] = {a2[0] - d * c0[0], a2[1] - d * c0[1], a2[2] - d * c0[2]};
    const double n2 = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (n2 > 1e-12) {
      for (int i = 0; i < 3; ++i) c1[i] = u[i] / n2;
    } else {  // any unit vector orthogonal to c0
      const double ax = fabs(c0[0]) < 0.9 ? 1.0 : 0.0, ay = 1.0 - ax;
      double v[3] = {ax - c0[0] * c0[0] * ax - c0[0] * c0[1] * ay, ay - c0[1] * c0[0] * ax - c0[1] * c0[1] * ay,
                     -c0[2] * (c0[0] * ax + c0[1] * ay)};
      const double nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
      for (int i = 0; i < 3; ++i) c1[i] = v[i] / nv;
    }
  }
  c2[0] = c0[1] * c1[2] - c0[2] * c1[1];
  c2[1] = c0[2] * c1[0] - c0[0] * c1[2];
  c2[2] = c0[0] * c1[1] - c0[1] * c1[0];
  const double* cs = cen + 3 * b;
  const double* ct = cen + 3 * (B + b);
  float* out = T + 16 * b;
  for (int i = 0; i < 3; ++i) {
    const double r0 = c0[i], r1 = c1[i], r2 = c2[i];
    out[4 * i + 0] = static_cast<float>(r0);
    out[4 * i + 1] = static_cast<float>(r1);
    out[4 * i + 2] = static_cast<float>(r2);
    out[4 * i + 3] = static_cast<float>(ct[i] + o[6 + i] / kScale - (r0 * cs[0] + r1 * cs[1] + r2 * cs[2]));
  }
  out[12] = out[13] = out[14] = 0.f;
  out[15] = 1.f;
}

// Row-major 4x4 source-to-target transforms -> training targets.
__global__ void k_labels(const float* __restrict__ T, const double* __restrict__ cen, int B, float* __restrict__ lab) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float* m = T + 16 * b;
  const double* cs = cen + 3 * b;
  const double* ct = cen + 3 * (B + b);
  float* l = lab + kOut * b;
  for (int i = 0; i < 3; ++i) {
    l[i] = m[4 * i + 0];
    l[3 + i] = m[4 * i + 1];
    const double rc = m[4 * i + 0] * cs[0] + m[4 * i + 1] * cs[1] + m[4 * i + 2] * cs[2];
    l[6 + i] = static_cast<float>((rc + m[4 * i + 3] - ct[i]) * kScale);
  }
}

}  // namespace

namespace posenet {

void head_forward(lcr_ctx* ctx, lcr_posenet* net, const Batch& b) {
  const int B = b.B;
  Epi e1;
  e1.bias = net->w + oC1;
  e1.relu = true;
  e1.outb = b.a1;
  e1.ldo = kH1;
  gemm_tc<256>(ctx, B, kH1, kIn, b.featb, net->pw.h1b, e1, net->err);
  Epi e2;
  e2.bias = net->w + oC2;
  e2.relu = true;
  e2.outb = b.a2;
  e2.ldo = kH2;
  gemm_tc<256>(ctx, B, kH2, kH1, b.a1, net->pw.h2b, e2, net->err);
  Epi e3;
  e3.bias = net->w + oC3;
  e3.out = b.y;
  e3.ldo = kOut;
  gemm_tc<16>(ctx, B, kOut, kH2, b.a2, net->pw.h3b, e3, net->err);
}

void loss_backward(lcr_ctx* ctx, lcr_posenet* net, const Batch& b) {
  const int B = b.B;
  float* g = net->grad;
  LCR_LAUNCH(ctx, k_loss, 1, 256, 0, b.y, b.labels, B, b.dy, b.loss);
  // head layer 3
  Epi eh3;
  eh3.out = g + oH3;
  eh3.ldo = kH2;
  gemm(ctx, kOut, kH2, B, b.dy, 1, kOut, b.a2, 1, kH2, eh3);
  LCR_LAUNCH(ctx, k_colsum, 1, 32, 0, b.dy, B, kOut, g + oC3);
  Epi ez2;
  ez2.mask = b.a2;
  ez2.ldm = kH2;
  ez2.out = b.dz2;
  ez2.ldo = kH2;
  gemm(ctx, B, kH2, kOut, b.dy, kOut, 1, net->pw.h3b, 1, kH2, ez2);
  // head layer 2
  Epi eh2;
  eh2.out = g + oH2;
  eh2.ldo = kH1;
  gemm(ctx, kH2, kH1, B, b.dz2, 1, kH2, b.a1, 1, kH1, eh2);
  LCR_LAUNCH(ctx, k_colsum, (kH2 + 127) / 128, 128, 0, b.dz2, B, kH2, g + oC2);
  Epi ez1;
  ez1.mask = b.a1;
  ez1.ldm = kH1;
  ez1.out = b.dz1;
  ez1.ldo = kH1;
  gemm(ctx, B, kH1, kH2, b.dz2, kH2, 1, net->pw.h2b, 1, kH1, ez1);
  // head layer 1
  Epi eh1;
  eh1.out = g + oH1;
  eh1.ldo = kIn;
  gemm(ctx, kH1, kIn, B, b.dz1, 1, kH1, b.featb, 1, kIn, eh1);
  LCR_LAUNCH(ctx, k_colsum, (kH1 + 127) / 128, 128, 0, b.dz1, B, kH1, g + oC1);
  Epi ex0;
  ex0.out = b.dx0;
  ex0.ldo = kIn;
  gemm(ctx, B, kIn, kH1, b.dz1, kH1, 1, net->pw.h1b, 1, kIn, ex0);
  // encoder
  LCR_LAUNCH(ctx, k_bwd_w3, kF3 / 8, 256, 0, b.feat, b.dx0, b.argmax, b.h2g, B, g);
  CUDA_TRY(cudaFuncSetAttribute(k_bwd_cloud, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kBwdSmem)));
  LCR_LAUNCH(ctx, k_bwd_cloud, 2 * B, 256, kBwdSmem, b.pts, b.feat, b.dx0, b.argmax, b.h2g, net->w, net->pw.w2b,
             net->pw.w3b, B, b.part);
  LCR_LAUNCH(ctx, k_reduce_part, (kEncLow + 255) / 256, 256, 0, b.part, 2 * B, g);
}

void adamw(lcr_ctx* ctx, lcr_posenet* net, const lcr_adamw_params* p) {
  net->step++;
  const float bc1 = static_cast<float>(1.0 - std::pow(static_cast<double>(p->beta1), static_cast<double>(net->step)));
  const float bc2 = static_cast<float>(1.0 - std::pow(static_cast<double>(p->beta2), static_cast<double>(net->step)));
  LCR_LAUNCH(ctx, k_adamw, 4 * ctx->sms, 256, 0, net->w, net->grad, net->m, net->v, p->lr, p->beta1, p->beta2,
             p->eps, p->weight_decay, bc1, bc2);
  pack(ctx, net);
}

void poses(lcr_ctx* ctx, const Batch& b) {
  if (b.B == 0) return;
  LCR_LAUNCH(ctx, k_poses, (b.B + 127) / 128, 128, 0, b.y, b.cen, b.B, b.guess);
}

void labels_from_poses(lcr_ctx* ctx, const Batch& b, const float* d_T) {
  if (b.B == 0) return;
  LCR_LAUNCH(ctx, k_labels, (b.B + 127) / 128, 128, 0, d_T, b.cen, b.B, b.labels);
}

}  // namespace posenet
