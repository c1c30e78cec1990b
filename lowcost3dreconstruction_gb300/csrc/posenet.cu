// Learned pose proposal: a shared-MLP point encoder and a pair head that
// predict a coarse rigid transform between two clouds, to replace the
// centroid_align guess (pcl_tools/centroid_align.cpp:102-130) in front of
// ICP (pcl_tools/fine_registration.cpp:105-126).
//
//   encoder  per point  p (3) -> 64 -> 128 -> 1024 (ReLU after each), max over
//            the 1024 points sampled from a cloud (centred on its centroid,
//            scaled by kScale) -> feature (1024)
//   head     [feature(src), feature(tgt)] (2048) -> 512 -> 256 -> 9
//            (ReLU after the first two): the first two columns of R (6) and
//            the residual translation delta (3), in the scaled frame, where
//            (q - c_tgt) = R (p - c_src) + delta.
//
// Weights and activations are bf16, accumulation fp32; the master weights,
// gradients and AdamW moments are fp32.  The encoder runs on the 5th-gen
// tensor cores: layer 1 (K=3) on the CUDA cores, layers 2 and 3 as tcgen05
// MMAs with TMEM accumulators, and the max-pool fused into the layer-3
// epilogue.  Layer 3 puts the channels on the MMA's M axis and the points on
// N, so each thread of the epilogue owns one channel and the max over points
// is a register reduction; nothing of the 1024-wide per-point activations
// ever reaches memory.  The head (0.6% of the flops at 1024 points per cloud)
// and the backward pass run on the CUDA cores in fixed summation orders, so
// every result is deterministic.
#include <cuda_bf16.h>

#include <cmath>

#include "posenet.cuh"
#include "tc.cuh"

using bf16 = __nv_bfloat16;

namespace {

using namespace posenet;

// ----------------------------------------------------------------- helpers
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// uniform in [0, 1) from the top 24 bits
__host__ __device__ __forceinline__ float u01(uint64_t h) { return static_cast<float>(h >> 40) * (1.0f / 16777216.0f); }

// ------------------------------------------------------------ parameters
// He-uniform weights, zero biases.
__global__ void k_init(float* __restrict__ w, uint64_t seed) {
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < kParams;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    int fan = 0;
    if (i < oB1) fan = 3;
    else if (i >= oW2 && i < oB2) fan = kF1;
    else if (i >= oW3 && i < oB3) fan = kF2;
    else if (i >= oH1 && i < oC1) fan = kIn;
    else if (i >= oH2 && i < oC2) fan = kH1;
    else if (i >= oH3 && i < oC3) fan = kH2;
    if (fan == 0) {
      w[i] = 0.f;
    } else {
      const float a = sqrtf(6.0f / static_cast<float>(fan));
      w[i] = (2.0f * u01(splitmix64(seed * 0x100000001b3ull + i)) - 1.0f) * a;
    }
  }
}

// bf16 copies of the weight matrices the kernels read: plain row-major ones and
// the swizzled shared-memory images of W2 (B operand of layer 2) and W3 (A
// operand of layer 3, one 32-KB image per 128-channel tile).
__global__ void k_pack(const float* __restrict__ w, PosenetWeights pw) {
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  const size_t i0 = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  for (size_t i = i0; i < static_cast<size_t>(kF2) * kF1; i += stride) {
    const int f = static_cast<int>(i / kF1), k = static_cast<int>(i % kF1);
    const bf16 v = __float2bfloat16_rn(w[oW2 + i]);
    pw.w2b[i] = v;
    *reinterpret_cast<bf16*>(pw.w2img + tc::sw128_offset(f, k, 128)) = v;
  }
  for (size_t i = i0; i < static_cast<size_t>(kF3) * kF2; i += stride) {
    const int c = static_cast<int>(i / kF2), k = static_cast<int>(i % kF2);
    const bf16 v = __float2bfloat16_rn(w[oW3 + i]);
    pw.w3b[i] = v;
    *reinterpret_cast<bf16*>(pw.w3img + (c >> 7) * kW3Tile + tc::sw128_offset(c & 127, k, 128)) = v;
  }
  for (size_t i = i0; i < static_cast<size_t>(kH1) * kIn; i += stride) pw.h1b[i] = __float2bfloat16_rn(w[oH1 + i]);
  for (size_t i = i0; i < static_cast<size_t>(kH2) * kH1; i += stride) pw.h2b[i] = __float2bfloat16_rn(w[oH2 + i]);
  for (size_t i = i0; i < static_cast<size_t>(kOut) * kH2; i += stride) pw.h3b[i] = __float2bfloat16_rn(w[oH3 + i]);
}

// ----------------------------------------------------------------- sample
// One block per cloud: FP64 centroid of the finite points (fixed-order block
// reduction), then kPts stratified samples, centred, scaled and rounded to
// bf16.  Sample i takes point floor((i + u_i) * n / kPts), u_i a hash of
// (seed, cloud, i); a non-finite point becomes the centroid.
__global__ void __launch_bounds__(256) k_sample(const CloudRef* __restrict__ clouds, uint64_t seed,
                                                float4* __restrict__ pts, double* __restrict__ cen) {
  __shared__ double red[4][256];
  const int cl = blockIdx.x, tid = threadIdx.x;
  const CloudRef c = clouds[cl];
  double sx = 0, sy = 0, sz = 0, sn = 0;
  for (long long i = tid; i < c.n; i += 256) {
    const float4 p = c.xyz[i];
    if (isfinite(p.x) && isfinite(p.y) && isfinite(p.z)) {
      sx += p.x;
      sy += p.y;
      sz += p.z;
      sn += 1.0;
    }
  }
  red[0][tid] = sx;
  red[1][tid] = sy;
  red[2][tid] = sz;
  red[3][tid] = sn;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (tid < s)
      for (int j = 0; j < 4; ++j) red[j][tid] += red[j][tid + s];
    __syncthreads();
  }
  const double cnt = red[3][0] > 0 ? red[3][0] : 1.0;
  const double cx = red[0][0] / cnt, cy = red[1][0] / cnt, cz = red[2][0] / cnt;
  if (tid == 0) {
    cen[cl * 3 + 0] = cx;
    cen[cl * 3 + 1] = cy;
    cen[cl * 3 + 2] = cz;
  }
  for (int i = tid; i < kPts; i += 256) {
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (c.n > 0) {
      const double u = u01(splitmix64(seed ^ (static_cast<uint64_t>(cl) << 32) ^ static_cast<uint64_t>(i)));
      long long j = static_cast<long long>((static_cast<double>(i) + u) * static_cast<double>(c.n) / kPts);
      j = j < c.n ? j : c.n - 1;
      const float4 p = c.xyz[j];
      if (isfinite(p.x) && isfinite(p.y) && isfinite(p.z)) {
        o.x = bf16r(static_cast<float>((p.x - cx) * kScale));
        o.y = bf16r(static_cast<float>((p.y - cy) * kScale));
        o.z = bf16r(static_cast<float>((p.z - cz) * kScale));
      }
    }
    pts[static_cast<size_t>(cl) * kPts + i] = o;
  }
}

// ---------------------------------------------------------------- encoder
// Shared-memory map of k_encode (offsets from a 1024-byte-aligned base).
constexpr uint32_t sW2 = 0;                    // W2 image, 128 x 64 bf16                      16 KB
constexpr uint32_t sA1 = sW2 + 16384;          // layer-1 output, 2 x (128 points x 64)        32 KB
constexpr uint32_t sB3 = sA1 + 32768;          // layer-2 output, 2 atoms x (256 points x 64)  64 KB
constexpr int kW3Ring = 3;                     // W3 tile images in flight
constexpr uint32_t sW3 = sB3 + 65536;          // W3 tile ring, 3 x 32 KB                      96 KB
constexpr uint32_t sRun = sW3 + kW3Ring * kW3Tile;  // running max per channel (f32)          4 KB
constexpr uint32_t sArg = sRun + 4 * kF3;      // its point (int)                               4 KB
constexpr uint32_t sW1 = sArg + 4 * kF3;       // (w0, w1, w2, b1) per layer-1 unit             1 KB
constexpr uint32_t sB2 = sW1 + 16 * kF1;       // b2                                          512 B
constexpr uint32_t sBar = sB2 + 4 * kF2;       // mbarriers (16 x 8 B), TMEM slot, flag
constexpr uint32_t kEncSmem = sBar + 160 + 1024;  // + alignment slack
static_assert(kEncSmem <= 227 * 1024, "encoder shared memory");
constexpr int kChunk = 256;                    // points per chunk (layer-2 M = 2 x 128)
constexpr int kGroupN = 256;                   // points per layer-3 MMA (N): the whole chunk
constexpr int kEpiThreads = 128;               // warps 0-3: layer 1, epilogues
constexpr int kEncThreads = kEpiThreads + 32;  // warp 4: bulk copies and MMA issue
// TMEM columns: layer-3 accumulators [0, 256) and [256, 512); layer 2's
// accumulator (two 128-point halves x 128 features) aliases the first one.
constexpr uint32_t kD2Col = 0;

// Barrier slots (uint64_t index from sBar).
enum : int {
  kBarW2 = 0,
  kBarW3Full = 1,    // [3]  tile image landed (bulk-copy bytes)
  kBarW3Empty = 4,   // [3]  MMAs reading the tile finished (MMA commit)
  kBarA1 = 7,        //      layer-1 operand written (128 arrivals)
  kBarD2 = 8,        //      layer-2 accumulator ready (MMA commit)
  kBarB3 = 9,        //      layer-3 operand written (128 arrivals)
  kBarD3Full = 10,   // [2]  layer-3 accumulator ready (MMA commit)
  kBarD3Empty = 12,  // [2]  layer-3 accumulator drained (128 arrivals)
  kBarDrain = 14,    //      every MMA issued so far completed (final commit)
  kBarCount = 15
};

// One CTA per SM encodes whole clouds one after the other, warp-specialised.
// Warps 0-3 (one thread per TMEM lane) compute layer 1 (3 -> 64) on the CUDA
// cores into the swizzled A operand of layer 2, move layer 2's accumulator
// (bias, ReLU, bf16) into the swizzled B operand of layer 3, and drain the
// layer-3 accumulators into the running max of their channel.  Warp 4 (one
// elected lane) keeps a ring of three W3 tile images filled by bulk copies and
// issues every MMA: layer 2 as two 128x128x64, layer 3 as eight
// 128(channels)x256(points)x128 per 256-point chunk into two TMEM buffers, so
// that the epilogue of one overlaps the MMA of the next (N = 256 halves the
// shared-memory operand bytes per flop against N = 128).  Layer 2 writes the
// first layer-3 buffer: it is issued after that buffer's last drain, and
// layer 3 of the chunk starts only after layer 2 was read (the B3 handoff).  Handoffs are
// mbarriers (MMA commits, bulk-copy byte counts, thread arrivals); every wait
// is bounded and a timeout drains what this CTA issued before its TMEM is
// freed.  kTrain also records the arg-max point per channel and stores the
// layer-2 activations for the backward pass.
template <bool kTrain>
__global__ void __launch_bounds__(kEncThreads, 1)
    k_encode(const float4* __restrict__ pts, int nclouds, int npairs, const float* __restrict__ w,
             const uint8_t* __restrict__ w2img, const uint8_t* __restrict__ w3img, float* __restrict__ feat,
             bf16* __restrict__ featb, int* __restrict__ argmax, bf16* __restrict__ h2g, int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const int tid = threadIdx.x, warp = tid >> 5;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + sBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + sBar + 8 * 16);
  volatile int* sflag = reinterpret_cast<volatile int*>(sm + sBar + 8 * 16 + 4);
  float* run = reinterpret_cast<float*>(sm + sRun);
  int* arg = reinterpret_cast<int*>(sm + sArg);
  float4* w1s = reinterpret_cast<float4*>(sm + sW1);
  float* b2s = reinterpret_cast<float*>(sm + sB2);

  const int ncl = (nclouds - static_cast<int>(blockIdx.x) + static_cast<int>(gridDim.x) - 1) / gridDim.x;
  const int nchunks = ncl * (kPts / kChunk);
  const int ntiles = nchunks * (kF3 / 128);
  if (tid == 0) {
    tc::mbar_init(&bar[kBarW2], 1);
    for (int i = 0; i < kW3Ring; ++i) {
      tc::mbar_init(&bar[kBarW3Full + i], 1);
      tc::mbar_init(&bar[kBarW3Empty + i], 1);
    }
    tc::mbar_init(&bar[kBarA1], kEpiThreads);
    tc::mbar_init(&bar[kBarD2], 1);
    tc::mbar_init(&bar[kBarB3], kEpiThreads);
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bar[kBarD3Full + i], 1);
      tc::mbar_init(&bar[kBarD3Empty + i], kEpiThreads);
    }
    tc::mbar_init(&bar[kBarDrain], 1);
    *sflag = 0;
    tc::mbar_fence_init();
  }
  for (int i = tid; i < kF1; i += kEncThreads)
    w1s[i] = make_float4(bf16r(w[oW1 + 3 * i]), bf16r(w[oW1 + 3 * i + 1]), bf16r(w[oW1 + 3 * i + 2]), w[oB1 + i]);
  for (int i = tid; i < kF2; i += kEncThreads) b2s[i] = w[oB2 + i];
  if (warp == 4) tc::tmem_alloc<512>(tslot);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 4) {
    // ================================================ bulk copies + MMA issue
    if ((tid & 31) == 0) {
      bool ok = true;
      int loaded = 0;      // tile images requested so far
      int tiles_used = 0;  // tile images whose MMAs were issued
      tc::mbar_expect_tx(&bar[kBarW2], 16384);
      tc::bulk_g2s(sm + sW2, w2img, 16384, &bar[kBarW2]);
      for (; loaded < kW3Ring && loaded < ntiles; ++loaded) {
        tc::mbar_expect_tx(&bar[kBarW3Full + loaded], kW3Tile);
        tc::bulk_g2s(sm + sW3 + loaded * kW3Tile, w3img + (loaded & 7) * kW3Tile, kW3Tile, &bar[kBarW3Full + loaded]);
      }
      ok = tc::mbar_wait(&bar[kBarW2], 0);
      const uint32_t id2 = tc::idesc_bf16_f32(128, 128), id3 = tc::idesc_bf16_f32(128, kGroupN);
      const uint32_t w2a = tc::smem_u32(sm + sW2), a1a = tc::smem_u32(sm + sA1), b3a = tc::smem_u32(sm + sB3);
      for (int C = 0; C < nchunks && ok && !*sflag; ++C) {
        // layer 2: D2[point][feature] for the two 128-point halves of the chunk,
        // into layer-3 buffer 0 once its last group (8C - 2) was drained
        if (!(ok = tc::mbar_wait(&bar[kBarA1], C & 1))) break;
        if (C > 0 && !(ok = tc::mbar_wait(&bar[kBarD3Empty], ((8 * C - 2) >> 1) & 1))) break;
        tc::tc_fence_after();
        for (int half = 0; half < 2; ++half)
          for (int s = 0; s < kF1 / 16; ++s)
            tc::mma_bf16(tmem + kD2Col + half * 128, tc::sdesc_sw128(a1a + half * 16384 + s * 32),
                         tc::sdesc_sw128(w2a + s * 32), id2, s > 0);
        tc::mma_commit(&bar[kBarD2]);
        // layer 3: one 256-point group per W3 tile, into alternating accumulators
        if (!(ok = tc::mbar_wait(&bar[kBarB3], C & 1))) break;
        tc::tc_fence_after();
        for (int ct = 0; ct < kF3 / 128 && ok; ++ct) {
          const int t = C * (kF3 / 128) + ct, rb = t % kW3Ring;
          if (!(ok = tc::mbar_wait(&bar[kBarW3Full + rb], (t / kW3Ring) & 1))) break;
          const uint32_t wa = tc::smem_u32(sm + sW3 + rb * kW3Tile);
          const int G = t, db = G & 1;
          if (G >= 2 && !(ok = tc::mbar_wait(&bar[kBarD3Empty + db], ((G - 2) >> 1) & 1))) break;
          tc::tc_fence_after();
          for (int s = 0; s < kF2 / 16; ++s)
            tc::mma_bf16(tmem + db * kGroupN, tc::sdesc_sw128(wa + (s >> 2) * 16384 + (s & 3) * 32),
                         tc::sdesc_sw128(b3a + (s >> 2) * (kChunk * 128) + (s & 3) * 32), id3, s > 0);
          tc::mma_commit(&bar[kBarD3Full + db]);
          tc::mma_commit(&bar[kBarW3Empty + rb]);
          tiles_used = t + 1;
          // refill the slot of the previous tile (its MMAs are done or nearly) two tiles ahead
          if (t >= 1 && loaded < ntiles) {
            const int pt = t - 1, pb = pt % kW3Ring;
            if (!(ok = tc::mbar_wait(&bar[kBarW3Empty + pb], (pt / kW3Ring) & 1))) break;
            tc::mbar_expect_tx(&bar[kBarW3Full + pb], kW3Tile);
            tc::bulk_g2s(sm + sW3 + pb * kW3Tile, w3img + (loaded & 7) * kW3Tile, kW3Tile, &bar[kBarW3Full + pb]);
            ++loaded;
          }
        }
      }
      if (!ok) *sflag = 1;
      // drain before the CTA's shared memory and TMEM go away: tile images requested but
      // never consumed (only after a failure), then one commit behind every MMA issued
      for (int t = tiles_used; t < loaded; ++t)
        tc::mbar_wait(&bar[kBarW3Full + t % kW3Ring], (t / kW3Ring) & 1);
      tc::mma_commit(&bar[kBarDrain]);
      if (!tc::mbar_wait(&bar[kBarDrain], 0)) *sflag = 1;
    }
  } else {
    // ======================================================== warps 0-3
    // Chunk C (global over this CTA's clouds) is cloud C / 4, points 256 (C % 4) ...
    // Layer 1 of chunk C+1 is computed right after chunk C's layer-3 operand is
    // handed over, so the MMA warp can queue layer 2 of C+1 behind layer 3 of C.
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    constexpr int kChunksPerCloud = kPts / kChunk;
    auto cloud_of = [&](int C) { return static_cast<int>(blockIdx.x) + (C / kChunksPerCloud) * static_cast<int>(gridDim.x); };
    // layer 1 (3 -> 64) of chunk C into the A operand of layer 2
    auto layer1 = [&](int C) {
      const size_t base = static_cast<size_t>(cloud_of(C)) * kPts + (C % kChunksPerCloud) * kChunk;
      for (int half = 0; half < 2; ++half) {
        const float4 p = pts[base + half * 128 + tid];
        unsigned char* A = sm + sA1 + half * 16384 + tid * 128;
#pragma unroll 1
        for (int c8 = 0; c8 < 8; ++c8) {
          uint32_t pk[4];
#pragma unroll
          for (int j2 = 0; j2 < 4; ++j2) {
            float h[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const float4 wv = w1s[c8 * 8 + j2 * 2 + e];
              float a = wv.w;
              a = fmaf(wv.x, p.x, a);
              a = fmaf(wv.y, p.y, a);
              a = fmaf(wv.z, p.z, a);
              h[e] = fmaxf(a, 0.f);
            }
            pk[j2] = pack_bf16x2(h[0], h[1]);
          }
          *reinterpret_cast<uint4*>(A + ((c8 ^ (tid & 7)) << 4)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
      tc::fence_async_smem();
      tc::tc_fence_before();
      tc::mbar_arrive(&bar[kBarA1]);
    };
    bool ok = true;
    for (int j = 0; j < kF3 / 128; ++j) {
      run[tid + 128 * j] = -INFINITY;
      arg[tid + 128 * j] = 0;
    }
    if (nchunks > 0) layer1(0);
    for (int C = 0; C < nchunks && ok; ++C) {
      const int cloud = cloud_of(C), pc = C % kChunksPerCloud;
      // ---- layer-2 epilogue into the B operand of layer 3 (free: chunk C-1's layer 3 completed)
      if (!(ok = tc::mbar_wait(&bar[kBarD2], C & 1))) break;
      tc::tc_fence_after();
      for (int half = 0; half < 2; ++half) {
        const int R = half * 128 + tid;  // point within the chunk
        float v[kF2];
        tc::tmem_ld128(tmem + lane_base + kD2Col + half * 128, v);
#pragma unroll
        for (int q = 0; q < kF2 / 32; ++q) {
#pragma unroll
          for (int c4 = 0; c4 < 4; ++c4) {
            uint32_t pk[4];
#pragma unroll
            for (int j2 = 0; j2 < 4; ++j2) {
              const int i0 = q * 32 + c4 * 8 + j2 * 2;
              pk[j2] = pack_bf16x2(fmaxf(v[i0] + b2s[i0], 0.f), fmaxf(v[i0 + 1] + b2s[i0 + 1], 0.f));
            }
            const int f0 = q * 32 + c4 * 8;
            const uint4 val = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            *reinterpret_cast<uint4*>(sm + sB3 + (f0 >> 6) * (kChunk * 128) + R * 128 +
                                      ((((f0 & 63) >> 3) ^ (R & 7)) << 4)) = val;
            if (kTrain)
              *reinterpret_cast<uint4*>(h2g + (static_cast<size_t>(cloud) * kPts + pc * kChunk + R) * kF2 + f0) = val;
          }
        }
      }
      tc::fence_async_smem();
      tc::tc_fence_before();
      tc::mbar_arrive(&bar[kBarB3]);
      // ---- layer 1 of the next chunk (A operand free: this chunk's layer 2 completed)
      if (C + 1 < nchunks) layer1(C + 1);
      // ---- layer-3 epilogues: the max over the chunk's 256 points, 128 columns at a time
      for (int ct = 0; ct < kF3 / 128 && ok; ++ct) {
        const int ch = ct * 128 + tid;
        float best = run[ch];
        int barg = arg[ch];
        const int G = C * (kF3 / 128) + ct, db = G & 1;
        if (!(ok = tc::mbar_wait(&bar[kBarD3Full + db], (G >> 1) & 1))) break;
        tc::tc_fence_after();
        for (int nh = 0; nh < 2; ++nh) {
          float v[128];
          tc::tmem_ld128(tmem + lane_base + db * kGroupN + nh * 128, v);
          if (nh == 1) {
            tc::tc_fence_before();
            tc::mbar_arrive(&bar[kBarD3Empty + db]);  // the values are in registers: release the buffer
          }
          if (kTrain) {
#pragma unroll
            for (int i = 0; i < 128; ++i)
              if (v[i] > best) {
                best = v[i];
                barg = pc * kChunk + nh * 128 + i;
              }
          } else {
            float m0 = v[0], m1 = v[1], m2 = v[2], m3 = v[3];  // four independent chains
#pragma unroll
            for (int i = 4; i < 128; i += 4) {
              m0 = fmaxf(m0, v[i]);
              m1 = fmaxf(m1, v[i + 1]);
              m2 = fmaxf(m2, v[i + 2]);
              m3 = fmaxf(m3, v[i + 3]);
            }
            best = fmaxf(best, fmaxf(fmaxf(m0, m1), fmaxf(m2, m3)));
          }
        }
        run[ch] = best;
        arg[ch] = barg;
      }
      if (*sflag) ok = false;
      if (!ok) break;
      if (pc == kChunksPerCloud - 1) {
        // ---- pooled feature: ReLU(max + b3); bias after the max (fp32 rounding is monotone)
        const int row = cloud < npairs ? cloud : cloud - npairs;
        const int col0 = cloud < npairs ? 0 : kF3;
        for (int j = 0; j < kF3 / 128; ++j) {
          const int c = tid + 128 * j;
          const float m = fmaxf(run[c] + w[oB3 + c], 0.f);
          feat[static_cast<size_t>(cloud) * kF3 + c] = m;
          featb[static_cast<size_t>(row) * kIn + col0 + c] = __float2bfloat16_rn(m);
          if (kTrain) argmax[static_cast<size_t>(cloud) * kF3 + c] = arg[c];
          run[c] = -INFINITY;
          arg[c] = 0;
        }
      }
    }
    if (!ok) *sflag = 1;
  }
  // ---- teardown
  tc::tc_fence_before();
  __syncthreads();
  if (*sflag && tid == 0) atomicExch(err, 1);
  if (warp == 4) {
    tc::tc_fence_after();
    tc::tmem_free<512>(tmem);
  }
}

}  // namespace

// ------------------------------------------------------------------- host
namespace posenet {

static size_t up(size_t x) { return (x + 1023) & ~static_cast<size_t>(1023); }

void create(lcr_ctx* ctx, lcr_posenet* net, uint64_t seed) {
  const size_t fb = up(kParams * sizeof(float));
  const size_t sizes[] = {fb, fb, fb, fb, 1024,
                          up(kF2 * kF1 * 2), up(static_cast<size_t>(kF3) * kF2 * 2), 16384, 8 * kW3Tile,
                          up(static_cast<size_t>(kH1) * kIn * 2), up(static_cast<size_t>(kH2) * kH1 * 2),
                          up(kOut * kH2 * 2)};
  size_t total = 0;
  for (size_t b : sizes) total += b;
  char* p = static_cast<char*>(dev_alloc(ctx, total));
  net->block = p;
  CUDA_TRY(cudaMemsetAsync(p, 0, total, ctx->stream));
  char* q = p;
  auto take = [&](size_t bytes) {
    char* r = q;
    q += bytes;
    return r;
  };
  net->w = reinterpret_cast<float*>(take(fb));
  net->grad = reinterpret_cast<float*>(take(fb));
  net->m = reinterpret_cast<float*>(take(fb));
  net->v = reinterpret_cast<float*>(take(fb));
  net->err = reinterpret_cast<int*>(take(1024));
  net->pw.w2b = reinterpret_cast<bf16*>(take(sizes[5]));
  net->pw.w3b = reinterpret_cast<bf16*>(take(sizes[6]));
  net->pw.w2img = reinterpret_cast<uint8_t*>(take(16384));
  net->pw.w3img = reinterpret_cast<uint8_t*>(take(8 * kW3Tile));
  net->pw.h1b = reinterpret_cast<bf16*>(take(sizes[9]));
  net->pw.h2b = reinterpret_cast<bf16*>(take(sizes[10]));
  net->pw.h3b = reinterpret_cast<bf16*>(take(sizes[11]));
  net->step = 0;
  LCR_LAUNCH(ctx, k_init, 2 * ctx->sms, 256, 0, net->w, seed);
  pack(ctx, net);
}

void destroy(lcr_ctx* ctx, lcr_posenet* net) {
  dev_free(ctx, net->block);
  dev_free(ctx, net->scratch);
  net->block = net->scratch = nullptr;
}

void pack(lcr_ctx* ctx, lcr_posenet* net) { LCR_LAUNCH(ctx, k_pack, 2 * ctx->sms, 256, 0, net->w, net->pw); }

Batch batch(lcr_ctx* ctx, lcr_posenet* net, int B, bool train) {
  const size_t C = 2 * static_cast<size_t>(B);
  const size_t sizes[] = {up(C * kPts * 16),      up(C * 3 * 8),       up(C * kF3 * 4),
                          up(B * kIn * 2ull),     up(C * kF3 * 4),     train ? up(C * kPts * kF2 * 2) : 0,
                          up(B * kH1 * 2ull),     up(B * kH2 * 2ull),  up(B * kOut * 4ull),
                          up(B * kOut * 4ull),    up(B * kOut * 4ull), up(B * kH2 * 4ull),
                          up(B * kH1 * 4ull),     up(B * kIn * 4ull),  train ? up(C * kEncLow * 4) : 0,
                          1024,                   up(C * sizeof(CloudRef)), up(B * 16 * 4ull)};
  size_t total = 0;
  for (size_t b : sizes) total += b;
  if (total > net->scratch_bytes) {
    dev_free(ctx, net->scratch);
    net->scratch = nullptr;
    net->scratch = dev_alloc(ctx, total);
    net->scratch_bytes = total;
  }
  char* q = static_cast<char*>(net->scratch);
  int i = 0;
  auto take = [&]() {
    char* r = q;
    q += sizes[i++];
    return r;
  };
  Batch b;
  b.B = B;
  b.pts = reinterpret_cast<float4*>(take());
  b.cen = reinterpret_cast<double*>(take());
  b.feat = reinterpret_cast<float*>(take());
  b.featb = reinterpret_cast<bf16*>(take());
  b.argmax = reinterpret_cast<int*>(take());
  b.h2g = reinterpret_cast<bf16*>(take());
  b.a1 = reinterpret_cast<bf16*>(take());
  b.a2 = reinterpret_cast<bf16*>(take());
  b.y = reinterpret_cast<float*>(take());
  b.labels = reinterpret_cast<float*>(take());
  b.dy = reinterpret_cast<float*>(take());
  b.dz2 = reinterpret_cast<float*>(take());
  b.dz1 = reinterpret_cast<float*>(take());
  b.dx0 = reinterpret_cast<float*>(take());
  b.part = reinterpret_cast<float*>(take());
  b.loss = reinterpret_cast<float*>(take());
  b.refs = reinterpret_cast<CloudRef*>(take());
  b.guess = reinterpret_cast<float*>(take());
  return b;
}

void sample(lcr_ctx* ctx, const CloudRef* d_refs, int nclouds, uint64_t seed, float4* pts, double* cen) {
  if (nclouds == 0) return;
  LCR_LAUNCH(ctx, k_sample, nclouds, 256, 0, d_refs, seed, pts, cen);
}

void encode(lcr_ctx* ctx, lcr_posenet* net, const Batch& b, bool train) {
  const int nclouds = 2 * b.B;
  if (nclouds == 0) return;
  CUDA_TRY(cudaFuncSetAttribute(k_encode<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kEncSmem));
  CUDA_TRY(cudaFuncSetAttribute(k_encode<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kEncSmem));
  const int grid = nclouds < ctx->sms ? nclouds : ctx->sms;
  KernelTimer kt(ctx, LCR_KT_ENCODE);
  if (train)
    LCR_LAUNCH(ctx, k_encode<true>, grid, kEncThreads, kEncSmem, b.pts, nclouds, b.B, net->w, net->pw.w2img, net->pw.w3img,
               b.feat, b.featb, b.argmax, b.h2g, net->err);
  else
    LCR_LAUNCH(ctx, k_encode<false>, grid, kEncThreads, kEncSmem, b.pts, nclouds, b.B, net->w, net->pw.w2img,
               net->pw.w3img, b.feat, b.featb, b.argmax, b.h2g, net->err);
}

void check_error(lcr_ctx* ctx, lcr_posenet* net) {
  int e = 0;
  CUDA_TRY(cudaMemcpyAsync(&e, net->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (e) {
    CUDA_TRY(cudaMemsetAsync(net->err, 0, sizeof(int), ctx->stream));
    LCR_THROW(LCR_ERR_TIMEOUT, "pose encoder: a bounded wait on the tensor-core pipeline expired");
  }
}

}  // namespace posenet
