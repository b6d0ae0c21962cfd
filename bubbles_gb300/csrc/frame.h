// frame.h -- device buffers and launcher of the particle-frame writer (frame.cu).
#pragma once

#include "bbg_kernels.h"

namespace bbg {

// SERIALIZER_* flags of the reference (src/third/serializer.h:7-14) this writer supports
constexpr int kFramePosition = 0x01;
constexpr int kFrameVelocity = 0x02;
constexpr int kFrameDensity = 0x04;
constexpr int kFrameMass = 0x20;
constexpr int kFrameSupported = kFramePosition | kFrameVelocity | kFrameDensity | kFrameMass;
constexpr int kFrameLineCap = 128;   // "\t\t" + 8 numbers of at most 12 characters + separators

struct FrameBufs {
    int capacity = 0;
    char *lines = nullptr;        // capacity x kFrameLineCap
    unsigned *lens = nullptr;     // capacity
    unsigned *scan_in = nullptr;  // capacity
    unsigned *offset = nullptr;   // capacity + 1
    unsigned *partials = nullptr;
    char *out = nullptr;          // capacity x kFrameLineCap
};

// Formats the particle lines of n particles (caller order through `slot`) and packs them
// into F.out; F.offset[n] is the byte count.
void launch_frame_lines(int n, int flags, const float4 *pos, const float4 *vel, const float *rho,
                        const int *slot, float mass, FrameBufs &F, cudaStream_t s);

}  // namespace bbg
