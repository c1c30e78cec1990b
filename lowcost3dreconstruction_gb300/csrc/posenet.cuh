// Learned pose proposal: shapes, parameter layout and device buffers shared by
// posenet.cu (sampling, encoder), posenet_train.cu (head, loss, backward,
// AdamW, training pairs) and the C ABI.
#pragma once

#include <cuda_bf16.h>

#include "lcr_internal.cuh"

namespace posenet {

constexpr int kPts = 1024;                   // points sampled per cloud
constexpr int kF1 = 64, kF2 = 128, kF3 = 1024;  // encoder widths
constexpr int kIn = 2 * kF3;                 // head input: [feature(src), feature(tgt)]
constexpr int kH1 = 512, kH2 = 256, kOut = 9;  // head widths; out = r6 (2 columns of R) + delta
constexpr float kScale = 4.0f;               // clouds are centred and scaled by 4 (1 / 0.25 m)
constexpr int kW3Tile = 128 * kF2 * 2;       // bytes of one 128-channel W3 tile image

// Flat fp32 parameter vector (row-major [out][in] matrices, then biases).
constexpr size_t oW1 = 0, oB1 = oW1 + kF1 * 3, oW2 = oB1 + kF1, oB2 = oW2 + kF2 * kF1, oW3 = oB2 + kF2,
                 oB3 = oW3 + static_cast<size_t>(kF3) * kF2, oH1 = oB3 + kF3, oC1 = oH1 + static_cast<size_t>(kH1) * kIn,
                 oH2 = oC1 + kH1, oC2 = oH2 + static_cast<size_t>(kH2) * kH1, oH3 = oC2 + kH2,
                 oC3 = oH3 + static_cast<size_t>(kOut) * kH2, kParams = oC3 + kOut;
static_assert(kParams == LCR_POSENET_PARAMS, "parameter count of the C ABI");
// Parameters whose per-cloud gradient partials the encoder backward writes: W1, b1, W2, b2.
constexpr int kEncLow = static_cast<int>(oW3 - oW1);

// bf16 copies of the weights, rebuilt from the fp32 master after every update.
struct PosenetWeights {
  __nv_bfloat16* w2b;   // [128][64]
  __nv_bfloat16* w3b;   // [1024][128]
  uint8_t* w2img;       // swizzled smem image of W2 (16 KB)
  uint8_t* w3img;       // 8 swizzled images of 128-channel W3 tiles (8 x 32 KB)
  __nv_bfloat16* h1b;   // [512][2048]
  __nv_bfloat16* h2b;   // [256][512]
  __nv_bfloat16* h3b;   // [9][256]
};

struct CloudRef {
  const float4* xyz;
  long long n;
};

}  // namespace posenet

struct lcr_posenet {
  float* w = nullptr;      // fp32 master parameters [kParams]
  float* grad = nullptr;   // gradients [kParams]
  float* m = nullptr;      // AdamW first moment
  float* v = nullptr;      // AdamW second moment
  int* err = nullptr;      // device error flag (a bounded wait expired)
  posenet::PosenetWeights pw{};
  void* block = nullptr;   // one allocation holding all of the above
  long long step = 0;      // AdamW steps taken
  // batch scratch, grown on demand
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
};

namespace posenet {

// Per-batch device buffers carved from lcr_posenet::scratch (B pairs, 2B clouds).
struct Batch {
  int B = 0;
  float4* pts;             // [2B][kPts] sampled, normalised points: src clouds, then tgt clouds
  double* cen;             // [2B][3] centroids
  float* feat;             // [2B][kF3] pooled features (fp32)
  __nv_bfloat16* featb;    // [B][kIn] head input
  int* argmax;             // [2B][kF3]
  __nv_bfloat16* h2g;      // [2B][kPts][kF2] layer-2 activations (training)
  __nv_bfloat16* a1;       // [B][kH1]
  __nv_bfloat16* a2;       // [B][kH2]
  float* y;                // [B][kOut]
  float* labels;           // [B][kOut]
  float* dy;               // [B][kOut]
  float* dz2;              // [B][kH2]
  float* dz1;              // [B][kH1]
  float* dx0;              // [B][kIn]
  float* part;             // [2B][kEncLow] per-cloud gradient partials
  float* loss;             // [1]
  CloudRef* refs;          // [2B]
  float* guess;            // [B][16]
};

Batch batch(lcr_ctx* ctx, lcr_posenet* net, int B, bool train);
void create(lcr_ctx* ctx, lcr_posenet* net, uint64_t seed);
void destroy(lcr_ctx* ctx, lcr_posenet* net);
void pack(lcr_ctx* ctx, lcr_posenet* net);
void sample(lcr_ctx* ctx, const CloudRef* d_refs, int nclouds, uint64_t seed, float4* pts, double* cen);
void encode(lcr_ctx* ctx, lcr_posenet* net, const Batch& b, bool train);
void head_forward(lcr_ctx* ctx, lcr_posenet* net, const Batch& b);
void loss_backward(lcr_ctx* ctx, lcr_posenet* net, const Batch& b);
void adamw(lcr_ctx* ctx, lcr_posenet* net, const lcr_adamw_params* p);
void poses(lcr_ctx* ctx, const Batch& b);
void labels_from_poses(lcr_ctx* ctx, const Batch& b, const float* d_T);
void check_error(lcr_ctx* ctx, lcr_posenet* net);

}  // namespace posenet
