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

// ---- reading (SerializerLoadParticles3) ----
constexpr int kFrameBoundary = 0x08;
constexpr int kFrameBoundaryExclusive = 0x100;
constexpr int kLineChunk = 16;                  // bytes per thread when finding line starts
constexpr int kPow5Lo = -500, kPow5Hi = 500;    // pow(5, e) table of the number reader
constexpr int kPow10Max = 400;                  // fraction digit weights 10^-r, r <= kPow10Max

// The first fluid section of a frame text, found on the host: its data lines are
// [data_begin, data_end) (data_end = start of the line holding "DataEnd").
struct FrameSection {
    size_t data_begin = 0, data_end = 0;
    int count = 0;     // the header's "Count"
    int flags = 0;     // from "Format" (or the caller's when absent)
};

// 0: found; 1: unknown format letter; 2: no fluid section or no "DataEnd"
int frame_find_section(const char *text, size_t length, int flags_in, FrameSection *out);

struct FrameReadBufs {
    size_t text_cap = 0, chunk_cap = 0, line_cap = 0;
    char *text = nullptr;
    unsigned *chunk = nullptr, *chunk_start = nullptr, *chunk_part = nullptr;
    unsigned *line = nullptr;                        // line start offsets
    float *vals = nullptr;                           // per line: position xyz, velocity xyz
    unsigned *valid = nullptr, *flag_copy = nullptr, *index = nullptr, *line_part = nullptr;
    double *pow5 = nullptr, *pow10 = nullptr;        // host libm values (the reference's)
};

// Line starts of F.text[0, bytes): returns the line count (synchronises).
cudaError_t frame_split_lines(size_t bytes, FrameReadBufs &F, unsigned *lines, unsigned *h_scratch,
                              cudaStream_t s);
// Parses every line (one thread per line) and numbers the particle lines; returns how many
// there are (synchronises).
cudaError_t frame_parse_lines(size_t bytes, unsigned lines, int flags, FrameReadBufs &F, unsigned *found,
                              unsigned *h_scratch, cudaStream_t s);
// Writes the first n particles' positions and velocities (xyz) to pos / vel.
void launch_frame_scatter(unsigned lines, int n, const FrameReadBufs &F, float *pos, float *vel,
                          cudaStream_t s);

}  // namespace bbg
