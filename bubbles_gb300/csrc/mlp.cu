// mlp.cu -- learned warm start of the PCISPH corrector.
//
// A per-particle MLP 4 -> 64 -> 64 -> 1 with GELU (tanh form) maps the features of a
// particle at the start of a substep to an estimate of its converged corrector pressure:
//   f0 = 100 (rho - rho0) / rho0                 local density error, percent
//   f1 = -100 dt div(v)                          compression rate (velocity divergence of the
//                                                previous substep's non-pressure pass)
//   f2 = (neighbours - 1) / 32                   neighbour count
//   f3 = p_prev / p_unit                         previous substep's converged pressure
// and the target is p / p_unit, with p_unit = delta * rho0 / 100 the pressure one
// corrector step assigns to a 1 % density error (delta of ComputeDelta), so the model
// does not depend on the substep length.
//
// Inference runs on the tensor cores: BF16 weights and activations, FP32 accumulation,
// mma.sync m16n8k16 (a warp evaluates 16 particles per pass: 8 MMAs for layer 1 with
// the bias folded in as a constant input, 32 for layer 2; layer 3 is a 64-term dot
// product on the FP32 pipes reduced across the quad).  Training is FP32 on the CUDA
// cores: one block of 128 samples per CTA computes the forward pass, back-propagates
// the squared error and reduces its weight gradients in shared memory; an Adam kernel
// updates the FP32 master parameters and rebuilds the BF16 fragments.
#include "bbg_kernels.h"
#include "mlp.h"

#include <algorithm>

#include <cuda_bf16.h>

namespace bbg {

namespace {

constexpr float kGeluC = 0.7978845608028654f;   // sqrt(2 / pi)
constexpr float kGeluA = 0.044715f;

// FP32 GELU and its derivative for training
__device__ __forceinline__ void gelu_grad(float x, float *y, float *dy) {
    const float x2 = x * x;
    const float u = kGeluC * fmaf(kGeluA * x2, x, x);
    const float th = tanhf(u);
    *y = 0.5f * x * (1.f + th);
    *dy = 0.5f * (1.f + th) + 0.5f * x * (1.f - th * th) * kGeluC * fmaf(3.f * kGeluA, x2, 1.f);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ __nv_bfloat162 as_bf2(uint32_t v) { return *reinterpret_cast<__nv_bfloat162 *>(&v); }
__device__ __forceinline__ uint32_t as_u32(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t *>(&v); }

// Inference folds GELU's constants into the weights.  With y = c x (c = sqrt(2 / pi)):
//   GELU(x) = 0.5 x (1 + tanh(c (x + a x^3))) = (0.5 / c) y (1 + tanh(y + (a / c^2) y^3)),
// so the packed layer 1 holds c W1, c b1 and yields y1; the hidden activation is
// h = y (1 + tanh(y + a' y^3)), a' = a / c^2; layer 2 holds 0.5 W2 (= c W2 (0.5 / c)) and
// c b2 and yields y2; layer 3 holds (0.5 / c) w3.
constexpr float kGeluAFold = kGeluA / (kGeluC * kGeluC);

// h = y (1 + tanh(y + a' y^3)) of two BF16 values in BF16 arithmetic: 5 paired operations,
// one of them on the MUFU pipe (tanh.approx.bf16x2).
__device__ __forceinline__ uint32_t gelu_bf16x2(uint32_t yv) {
    const __nv_bfloat162 y = as_bf2(yv);
    const __nv_bfloat162 a = __float2bfloat162_rn(kGeluAFold);
    const __nv_bfloat162 ay2 = __hmul2(__hmul2(y, y), a);
    const __nv_bfloat162 u = __hfma2(ay2, y, y);
    uint32_t t;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(t) : "r"(as_u32(u)));
    return as_u32(__hfma2(y, as_bf2(t), y));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Layer 1 input row of one particle as the A-fragment pair of lane quad position t:
// columns (2t, 2t+1) of [f0 f1 f2 f3 1 0 0 0 | 0 ...].
__device__ __forceinline__ uint32_t layer1_a(float4 f, int t) {
    switch (t) {
        case 0: return pack_bf16(f.x, f.y);
        case 1: return pack_bf16(f.z, f.w);
        case 2: return pack_bf16(1.f, 0.f);
        default: return 0u;
    }
}

}  // namespace

// Per-particle features at the start of a substep, right after the density pass (vel.w =
// 1 / rho); the divergence is the previous substep's sum (its non-pressure pass), carried
// through the grid rebuild, so the warm start can precede this substep's force pass.
__global__ void k_mlp_features(int n, const float4 *__restrict__ vel, const float *__restrict__ divsum,
                               const int *__restrict__ nbr, const float *__restrict__ pprev,
                               float4 *__restrict__ feat, float inv_rho0, float div_scale,
                               float inv_p_unit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float rho = 1.f / vel[i].w;
    feat[i] = make_float4(100.f * (rho * inv_rho0 - 1.f), div_scale * divsum[i],
                          (float)(nbr[i] - 1) * (1.f / 32.f), pprev[i] * inv_p_unit);
}

// Tensor-core inference fused with the warm start of the corrector: p = scale * p_unit *
// clamp(MLP(features), 0, largest training target), rho* = rho, err = 0, pos.w = p / rho^2.
// Layer-2 B fragments live in shared memory (8 KB per block), the layer-1 fragments,
// bias and w3 in registers; GELU runs in BF16x2 arithmetic.
__global__ void __launch_bounds__(128, kMlpBlocksPerSm)
k_mlp_warm_start(int n, const float4 *__restrict__ feat, const uint32_t *__restrict__ w1f,
                 const uint32_t *__restrict__ w2f, const float *__restrict__ tail, float p_unit, float scale,
                 float4 *__restrict__ pos, const float *__restrict__ rho, float *__restrict__ press,
                 float *__restrict__ rhostar, float *__restrict__ derr, float *__restrict__ raw) {
    __shared__ uint2 sW2[32 * 32];   // [fragment pair q / 2][lane]
    __shared__ float2 sB2[32], sW3[32];   // (b2, w3) column pairs 2p, 2p + 1
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    for (int k = threadIdx.x; k < 32 * 32; k += blockDim.x) {
        const int qp = k >> 5, l = k & 31;
        sW2[k] = make_uint2(__ldg(&w2f[(2 * qp) * 32 + l]), __ldg(&w2f[(2 * qp + 1) * 32 + l]));
    }
    if (threadIdx.x < 32) {
        const int c = 2 * threadIdx.x;
        sB2[threadIdx.x] = make_float2(__ldg(&tail[kTailB2 + c]), __ldg(&tail[kTailB2 + c + 1]));
        sW3[threadIdx.x] = make_float2(__ldg(&tail[kTailW3 + c]), __ldg(&tail[kTailW3 + c + 1]));
    }
    uint32_t b1f[8];
#pragma unroll
    for (int q = 0; q < 8; q++) b1f[q] = __ldg(&w1f[q * 32 + lane]);
    const float b3 = __ldg(&tail[kTailB3]);
    const float ymax = __ldg(&tail[kTailYmax]);
    __syncthreads();
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 16; base < n; base += warps * 16) {
        const int pa = base + g, pb = base + g + 8;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 fa = pa < n ? __ldg(&feat[pa]) : z4;
        const float4 fb = pb < n ? __ldg(&feat[pb]) : z4;
        const uint32_t a0 = layer1_a(fa, t), a1 = layer1_a(fb, t);
        // layer 1: 16 x 16 (features, bias) times 16 x 64
        uint32_t h1[16];   // bf16 pairs, A fragments of layer 2 (4 k-chunks x 4 regs)
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            mma_bf16(c, a0, a1, 0u, 0u, b1f[nt], 0u);
            const int kc = nt >> 1, hi = nt & 1;
            h1[kc * 4 + hi * 2 + 0] = gelu_bf16x2(pack_bf16(c[0], c[1]));
            h1[kc * 4 + hi * 2 + 1] = gelu_bf16x2(pack_bf16(c[2], c[3]));
        }
        // layer 2 (16 x 64 times 64 x 64, accumulators starting at the bias) and layer 3 on the
        // FP32 pipes (rows g: c0, c1 and g + 8: c2, c3), in two halves of 32 output columns so
        // that half the accumulators are live at a time
        float ya = 0.f, yb = 0.f;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float acc[4][4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 b = sB2[4 * (4 * half + q) + t];   // columns 8 nt + 2 t, + 1
                acc[q][0] = b.x;
                acc[q][1] = b.y;
                acc[q][2] = b.x;
                acc[q][3] = b.y;
            }
#pragma unroll
            for (int kc = 0; kc < 4; kc++) {
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const uint2 bf = sW2[(kc * 8 + 4 * half + q) * 32 + lane];
                    mma_bf16(acc[q], h1[kc * 4 + 0], h1[kc * 4 + 1], h1[kc * 4 + 2], h1[kc * 4 + 3], bf.x, bf.y);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 w = sW3[4 * (4 * half + q) + t];
                const float2 ha = __bfloat1622float2(as_bf2(gelu_bf16x2(pack_bf16(acc[q][0], acc[q][1]))));
                const float2 hb = __bfloat1622float2(as_bf2(gelu_bf16x2(pack_bf16(acc[q][2], acc[q][3]))));
                ya = fmaf(ha.x, w.x, ya);
                ya = fmaf(ha.y, w.y, ya);
                yb = fmaf(hb.x, w.x, yb);
                yb = fmaf(hb.y, w.y, yb);
            }
        }
        ya += __shfl_xor_sync(0xffffffffu, ya, 1);
        ya += __shfl_xor_sync(0xffffffffu, ya, 2);
        yb += __shfl_xor_sync(0xffffffffu, yb, 1);
        yb += __shfl_xor_sync(0xffffffffu, yb, 2);
        const int p_out = t == 0 ? pa : pb;
        const float y = (t == 0 ? ya : yb) + b3;
        if (t < 2 && p_out < n) {
            if (raw) raw[p_out] = y;
            if (press) {
                float e = fmaxf(y, 0.f);
                if (ymax > 0.f) e = fminf(e, ymax);
                const float p = scale * p_unit * e;
                const float d = rho[p_out];
                press[p_out] = p;
                rhostar[p_out] = d;
                derr[p_out] = 0.f;
                reinterpret_cast<float *>(&pos[p_out])[3] = p / (d * d);
            }
        }
    }
}

// Training pairs of the substep that just converged: features at its start and the
// converged pressure / p_unit, B particles spread evenly over the slots from a per-step
// offset; the largest target seen bounds the estimates of inference.
__global__ void k_mlp_collect(int n, int batch, const unsigned *__restrict__ step,
                              const float4 *__restrict__ feat, const float *__restrict__ press,
                              float inv_p_unit, float4 *__restrict__ bx, float *__restrict__ bt,
                              float *ymax) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= batch) return;
    const unsigned s = *step;
    const unsigned long long off = (unsigned long long)((s * 2654435761u) % (unsigned)n);
    const int i = (int)((off + (unsigned long long)b * (unsigned long long)n / (unsigned long long)batch) %
                        (unsigned long long)n);
    bx[b] = feat[i];
    const float y = press[i] * inv_p_unit;
    bt[b] = y;
    if (y > 0.f) atomicMax(reinterpret_cast<unsigned *>(ymax), __float_as_uint(y));
}

// Forward + backward of 128-sample tiles (tile, tile + gridDim.x, ...): each block sums
// its tiles' weight gradients into its own row of gpart and their (weighted) squared
// errors into lpart[block], always in the same order, so training is deterministic (no
// atomics; the Adam kernel adds the rows in block order).
__global__ void __launch_bounds__(128)
k_mlp_train(int batch, const float4 *__restrict__ bx, const float *__restrict__ bt,
            const float *__restrict__ theta, float *__restrict__ gpart, double *__restrict__ lpart,
            float expectile) {
    extern __shared__ float smem[];
    float *sW2 = smem;                    // [64][64]
    float *sW1 = sW2 + kHid * kHid;       // [4][64]
    float *sB1 = sW1 + kIn * kHid;        // [64]
    float *sB2 = sB1 + kHid;              // [64]
    float *sW3 = sB2 + kHid;              // [64]
    float *sX = sW3 + kHid;               // [4][128]
    float *sH1 = sX + kIn * 128;          // [64][128]
    float *sD1 = sH1 + kHid * 128;        // [64][128]
    float *sH2 = sD1 + kHid * 128;        // [64][128]
    float *sD2 = sH2 + kHid * 128;        // [64][128]
    float *sDY = sD2 + kHid * 128;        // [128]
    __shared__ double sLoss[4];
    const int t = threadIdx.x;
    for (int k = t; k < kHid * kHid; k += 128) sW2[k] = theta[kOffW2 + k];
    for (int k = t; k < kIn * kHid; k += 128) sW1[k] = theta[kOffW1 + k];
    if (t < kHid) {
        sB1[t] = theta[kOffB1 + t];
        sB2[t] = theta[kOffB2 + t];
        sW3[t] = theta[kOffW3 + t];
    }
    __syncthreads();
    const float b3 = theta[kOffB3];
    float *grad = gpart + (size_t)blockIdx.x * kParams;
    for (int tile = blockIdx.x; tile * 128 < batch; tile += gridDim.x) {
        const bool first = tile == (int)blockIdx.x;
        // a block's own gradient row: the first tile stores, later tiles add (same thread)
        auto put = [&](int idx, float v) { grad[idx] = first ? v : grad[idx] + v; };
        const int s = tile * 128 + t;
        const bool valid = s < batch;
        const float4 x = valid ? bx[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float target = valid ? bt[s] : 0.f;
        sX[0 * 128 + t] = x.x;
        sX[1 * 128 + t] = x.y;
        sX[2 * 128 + t] = x.z;
        sX[3 * 128 + t] = x.w;
        // forward
        for (int a = 0; a < kHid; a++) {
            float z = sB1[a];
            z = fmaf(x.x, sW1[0 * kHid + a], z);
            z = fmaf(x.y, sW1[1 * kHid + a], z);
            z = fmaf(x.z, sW1[2 * kHid + a], z);
            z = fmaf(x.w, sW1[3 * kHid + a], z);
            float h, d;
            gelu_grad(z, &h, &d);
            sH1[a * 128 + t] = h;
            sD1[a * 128 + t] = d;
        }
        float z2[kHid];
    #pragma unroll
        for (int k = 0; k < kHid; k++) z2[k] = sB2[k];
        for (int a = 0; a < kHid; a++) {
            const float h = sH1[a * 128 + t];
    #pragma unroll
            for (int k = 0; k < kHid; k++) z2[k] = fmaf(h, sW2[a * kHid + k], z2[k]);
        }
        float y = b3;
    #pragma unroll
        for (int k = 0; k < kHid; k++) {
            float h, d;
            gelu_grad(z2[k], &h, &d);
            sH2[k * 128 + t] = h;
            y = fmaf(sW3[k], h, y);
            z2[k] = d;   // keep GELU'(z2)
        }
        const float err = valid ? y - target : 0.f;
        // asymmetric squared error (expectile tau): over-estimates weigh (1 - tau) / 0.5,
        // under-estimates tau / 0.5; tau = 0.5 is the mean squared error
        const float wgt = (err > 0.f ? 1.f - expectile : expectile) * 2.f;
        const float dy = 2.f * wgt * err / (float)batch;
        sDY[t] = dy;
        // backward through layer 3 and GELU 2
    #pragma unroll
        for (int k = 0; k < kHid; k++) {
            z2[k] = dy * sW3[k] * z2[k];   // dz2
            sD2[k * 128 + t] = z2[k];
        }
        // backward through layer 2 and GELU 1
        for (int a = 0; a < kHid; a++) {
            float acc = 0.f;
    #pragma unroll
            for (int k = 0; k < kHid; k++) acc = fmaf(sW2[a * kHid + k], z2[k], acc);
            sD1[a * 128 + t] *= acc;   // dz1
        }
        // squared error of the block
        double l = (double)wgt * (double)err * (double)err;
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((t & 31) == 0) sLoss[t >> 5] = l;
        __syncthreads();
        if (t == 0) {
            const double bl = sLoss[0] + sLoss[1] + sLoss[2] + sLoss[3];
            lpart[blockIdx.x] = first ? bl : lpart[blockIdx.x] + bl;
        }
        // dW2[a][k] = sum_s h1[a][s] dz2[k][s]: thread -> row a = t / 2, 32 columns
        {
            const int a = t >> 1, k0 = (t & 1) * 32;
            float acc[32];
    #pragma unroll
            for (int kk = 0; kk < 32; kk++) acc[kk] = 0.f;
            for (int q = 0; q < 128; q++) {
                const float h = sH1[a * 128 + q];
    #pragma unroll
                for (int kk = 0; kk < 32; kk++) acc[kk] = fmaf(h, sD2[(k0 + kk) * 128 + q], acc[kk]);
            }
    #pragma unroll
            for (int kk = 0; kk < 32; kk++) put(kOffW2 + a * kHid + k0 + kk, acc[kk]);
        }
        // dW1[f][a] = sum_s x[f][s] dz1[a][s]: thread -> a = t / 2, f = 2 (t & 1) + {0, 1}
        {
            const int a = t >> 1, f0 = (t & 1) * 2;
            float g0 = 0.f, g1 = 0.f;
            for (int q0 = 0; q0 < 128; q0++) {
                const int q = (q0 + t) & 127;
                const float d = sD1[a * 128 + q];
                g0 = fmaf(sX[f0 * 128 + q], d, g0);
                g1 = fmaf(sX[(f0 + 1) * 128 + q], d, g1);
            }
            put(kOffW1 + f0 * kHid + a, g0);
            put(kOffW1 + (f0 + 1) * kHid + a, g1);
        }
        // bias and layer-3 gradients: rows summed with a rotated start (no bank conflicts)
        if (t < kHid) {
            float gb2 = 0.f, gw3 = 0.f;
            for (int q0 = 0; q0 < 128; q0++) {
                const int q = (q0 + t) & 127;
                gb2 += sD2[t * 128 + q];
                gw3 = fmaf(sH2[t * 128 + q], sDY[q], gw3);
            }
            put(kOffB2 + t, gb2);
            put(kOffW3 + t, gw3);
        } else {
            const int a = t - kHid;
            float gb1 = 0.f;
            for (int q0 = 0; q0 < 128; q0++) gb1 += sD1[a * 128 + ((q0 + t) & 127)];
            put(kOffB1 + a, gb1);
        }
        if (t < 32) {
            float gb3 = sDY[t] + sDY[t + 32] + sDY[t + 64] + sDY[t + 96];
            for (int o = 16; o > 0; o >>= 1) gb3 += __shfl_xor_sync(0xffffffffu, gb3, o);
            if (t == 0) put(kOffB3, gb3);
        }
        __syncthreads();   // the tile's shared rows are rewritten by the next tile
    }
}

// Adam on the FP32 master parameters (bias corrections from the device step counter); the
// gradient is the sum of the training blocks' rows in block order, the batch loss the sum
// of their partial losses in block order.
__global__ void k_mlp_adam(float *__restrict__ theta, const float *__restrict__ gpart, int rows,
                           const double *__restrict__ lpart, double *__restrict__ loss, float *__restrict__ m1,
                           float *__restrict__ m2, const unsigned *__restrict__ step, float lr, float beta1,
                           float beta2, float eps) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        double l = 0.0;
        for (int b = 0; b < rows; b++) l += lpart[b];
        *loss += l;
    }
    if (p >= kParams) return;
    float gr = 0.f;
    for (int b = 0; b < rows; b++) gr += gpart[(size_t)b * kParams + p];
    const float a = beta1 * m1[p] + (1.f - beta1) * gr;
    const float b = beta2 * m2[p] + (1.f - beta2) * gr * gr;
    m1[p] = a;
    m2[p] = b;
    const float tstep = (float)(*step + 1u);
    const float c1 = 1.f / (1.f - powf(beta1, tstep));
    const float c2 = 1.f / (1.f - powf(beta2, tstep));
    theta[p] -= lr * (a * c1) / (sqrtf(b * c2) + eps);
}

// BF16 B fragments of the tensor-core layers and the FP32 tail from the master
// parameters; advances the training step counter.
__global__ void k_mlp_pack(const float *__restrict__ theta, uint32_t *__restrict__ w1f,
                           uint32_t *__restrict__ w2f, float *__restrict__ tail, unsigned *step, int advance) {
    const int tid = threadIdx.x;   // one block of 256 threads
    // layer 1: [W1 (rows 0-3); b1 (row 4); 0] as 16 x 64, lane's b0 of n-tile nt
    for (int k = tid; k < 8 * 32; k += blockDim.x) {
        const int nt = k / 32, lane = k % 32, g = lane >> 2, t = lane & 3;
        const int col = 8 * nt + g;
        auto w1 = [&](int r) -> float {   // c W1, c b1 (the folded GELU)
            if (r < kIn) return kGeluC * theta[kOffW1 + r * kHid + col];
            if (r == kIn) return kGeluC * theta[kOffB1 + col];
            return 0.f;
        };
        w1f[k] = pack_bf16(w1(2 * t), w1(2 * t + 1));
    }
    // layer 2: W2 [64 (k)][64 (n)], fragments (k-chunk kc, n-tile nt, half hh)
    for (int k = tid; k < 64 * 32; k += blockDim.x) {
        const int q = k / 32, lane = k % 32, g = lane >> 2, t = lane & 3;
        const int kc = q / 16, nt = (q / 2) % 8, hh = q & 1;
        const int row = 16 * kc + 8 * hh + 2 * t, col = 8 * nt + g;
        w2f[k] = pack_bf16(0.5f * theta[kOffW2 + row * kHid + col], 0.5f * theta[kOffW2 + (row + 1) * kHid + col]);
    }
    for (int k = tid; k < kHid; k += blockDim.x) {
        tail[kTailB2 + k] = kGeluC * theta[kOffB2 + k];
        tail[kTailW3 + k] = __bfloat162float(__float2bfloat16_rn((0.5f / kGeluC) * theta[kOffW3 + k]));
    }
    if (tid == 0) {
        tail[kTailB3] = theta[kOffB3];
        if (advance) *step += 1u;
    }
}

// ----------------------------------------------------------------------------
// launchers
// ----------------------------------------------------------------------------
static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

void launch_mlp_features(const Params &P, const DevBufs &B, const MlpBufs &M, int buf, float dt,
                         float p_unit, cudaStream_t s) {
    // div = m * spiky_dw_c * divsum (non-pressure pass); f1 = -100 dt div
    const float div_scale = -100.f * dt * P.mass * P.spiky_dw_c;
    k_mlp_features<<<blocks_for(P.n, 256), 256, 0, s>>>(P.n, B.vel[buf], M.divprev, B.nbr, B.pprev, M.feat,
                                                         1.f / P.target_density, div_scale, 1.f / p_unit);
}

void launch_mlp_warm_start(const Params &P, const DevBufs &B, const MlpBufs &M, int buf, float p_unit,
                           float scale, cudaStream_t s) {
    BBG_PBEGIN(B, KID_MLP, s, -1);
    const int warps = (P.n + 15) / 16;
    int blocks = (warps + 3) / 4;
    if (blocks > M.infer_blocks) blocks = M.infer_blocks;
    if (blocks < 1) blocks = 1;
    k_mlp_warm_start<<<blocks, 128, 0, s>>>(P.n, M.feat, M.w1f, M.w2f, M.tail, p_unit, scale, B.pos[buf],
                                            B.rho, B.press, B.rhostar, B.derr, nullptr);
    BBG_PEND(B, s);
}

void launch_mlp_infer_raw(const MlpBufs &M, const float4 *feat, int n, float *out, cudaStream_t s) {
    const int warps = (n + 15) / 16;
    int blocks = (warps + 3) / 4;
    if (blocks > M.infer_blocks) blocks = M.infer_blocks;
    if (blocks < 1) blocks = 1;
    k_mlp_warm_start<<<blocks, 128, 0, s>>>(n, feat, M.w1f, M.w2f, M.tail, 1.f, 1.f, nullptr, nullptr,
                                            nullptr, nullptr, nullptr, out);
}

size_t mlp_train_smem() {
    return sizeof(float) * ((size_t)kHid * kHid + kIn * kHid + 3 * kHid + kIn * 128 + 4 * kHid * 128 + 128);
}

cudaError_t mlp_prepare() {
    return cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mlp_train_smem());
}

void launch_mlp_train_step(const MlpBufs &M, const float4 *bx, const float *bt, int batch, float lr,
                           float beta1, float beta2, float eps, float expectile, cudaStream_t s) {
    const int rows = std::min(blocks_for(batch, 128), kGradRows);
    k_mlp_train<<<rows, 128, mlp_train_smem(), s>>>(batch, bx, bt, M.theta, M.grad, M.lpart, expectile);
    k_mlp_adam<<<blocks_for(kParams, 256), 256, 0, s>>>(M.theta, M.grad, rows, M.lpart, M.loss, M.m1, M.m2,
                                                         M.step, lr, beta1, beta2, eps);
    k_mlp_pack<<<1, 256, 0, s>>>(M.theta, M.w1f, M.w2f, M.tail, M.step, 1);
}

void launch_mlp_collect(const Params &P, const DevBufs &B, const MlpBufs &M, float p_unit, cudaStream_t s) {
    k_mlp_collect<<<blocks_for(M.batch, 256), 256, 0, s>>>(P.n, M.batch, M.step, M.feat, B.press,
                                                           1.f / p_unit, M.bx, M.bt, M.tail + kTailYmax);
}

__global__ void k_mlp_get_features(const float4 *__restrict__ feat, const int *__restrict__ slot, float *out,
                                   int n) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const float4 f = feat[slot[id]];
    out[4 * id] = f.x;
    out[4 * id + 1] = f.y;
    out[4 * id + 2] = f.z;
    out[4 * id + 3] = f.w;
}

void launch_mlp_get_features(const MlpBufs &M, const int *slot, float *out, int n, cudaStream_t s) {
    k_mlp_get_features<<<blocks_for(n, 256), 256, 0, s>>>(M.feat, slot, out, n);
}

void launch_mlp_pack(const MlpBufs &M, cudaStream_t s) {
    k_mlp_pack<<<1, 256, 0, s>>>(M.theta, M.w1f, M.w2f, M.tail, M.step, 0);
}

}  // namespace bbg
