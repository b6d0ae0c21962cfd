// mlp.h -- buffers and launchers of the learned corrector warm start (mlp.cu).
#pragma once

#include "bbg_kernels.h"

#include <stdint.h>

namespace bbg {

constexpr int kIn = 4, kHid = 64;
// FP32 master parameters: W1 [4][64], b1 [64], W2 [64][64], b2 [64], w3 [64], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kHid;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid;
constexpr int kParams = kOffB3 + 1;
// FP32 tail used by inference: b2 [64], w3 [64] (rounded to BF16), b3, and the largest
// training target (estimates are clamped to it; 0 = no bound)
constexpr int kTailB2 = 0, kTailW3 = kHid, kTailB3 = 2 * kHid, kTailYmax = 2 * kHid + 1;
constexpr int kTail = 2 * kHid + 2;
constexpr int kGradRows = 128;   // training blocks (each loops over 128-sample tiles)

struct MlpBufs {
    float *theta = nullptr, *m1 = nullptr, *m2 = nullptr;   // kParams each
    float *grad = nullptr;     // kGradRows x kParams: per-block gradient rows of a training step
    double *lpart = nullptr;   // kGradRows: per-block losses of a training step
    uint32_t *w1f = nullptr;   // 8 x 32 BF16x2 B fragments of [W1; b1]
    uint32_t *w2f = nullptr;   // 64 x 32 BF16x2 B fragments of W2
    float *tail = nullptr;     // kTail
    unsigned *step = nullptr;  // Adam steps taken
    double *loss = nullptr;    // sum of squared errors of the training batches
    float4 *feat = nullptr;    // per-particle features (sorted slots)
    float *divsum = nullptr;   // velocity-divergence sum of this substep's non-pressure pass
    float *divprev = nullptr;  // the previous substep's, carried into the current order
    float4 *bx = nullptr;      // training batch: features
    float *bt = nullptr;       //                 targets (pressure / p_unit)
    int batch = 0;
    int infer_blocks = 1;      // persistent inference grid
};

#ifndef BBG_MLP_MIN_BLOCKS
#define BBG_MLP_MIN_BLOCKS 8
#endif
// resident 128-thread blocks per SM of the inference kernel (its register budget; build-time
// tuning knob) and the size of its persistent grid per SM
constexpr int kMlpBlocksPerSm = BBG_MLP_MIN_BLOCKS;

cudaError_t mlp_prepare();
void launch_mlp_features(const Params &P, const DevBufs &B, const MlpBufs &M, int buf, float dt,
                         float p_unit, cudaStream_t s);
void launch_mlp_warm_start(const Params &P, const DevBufs &B, const MlpBufs &M, int buf, float p_unit,
                           float scale, cudaStream_t s);
// raw network outputs (pressure / p_unit before the clamp) for n host-provided features
void launch_mlp_infer_raw(const MlpBufs &M, const float4 *feat, int n, float *out, cudaStream_t s);
// one forward / backward / Adam step on a batch, then the BF16 fragments are rebuilt
void launch_mlp_train_step(const MlpBufs &M, const float4 *bx, const float *bt, int batch, float lr,
                           float beta1, float beta2, float eps, float expectile, cudaStream_t s);
void launch_mlp_collect(const Params &P, const DevBufs &B, const MlpBufs &M, float p_unit, cudaStream_t s);
void launch_mlp_pack(const MlpBufs &M, cudaStream_t s);
// features in caller order (n x 4 floats) through the id -> slot map
void launch_mlp_get_features(const MlpBufs &M, const int *slot, float *out, int n, cudaStream_t s);

}  // namespace bbg
