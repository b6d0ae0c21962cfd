// frame.cu -- particle frames in the reference's text format, formatted on the device.
//
// SerializerSaveSphDataSet3 (src/third/serializer.cpp:880-923) appends a block
//   FluidBegin / "Type" particles / "Count" n / "Format" <flags> / "Spacing" h0 /
//   DataBegin / one line per particle / DataEnd / FluidEnd
// where each particle line is two tabs, the selected fields as %g numbers separated by
// spaces (position, velocity, density, mass; PushParticleSetToFile, :824-878) and a newline.
// Here one thread formats one particle's line (caller order) into a fixed-size slot with
// the exact %g of gfmt.h, an exclusive scan of the line lengths gives each line's offset,
// and a second pass packs the lines into one contiguous buffer: the host receives only the
// bytes of the frame.
#include "bbg_kernels.h"
#include "frame.h"
#include "gfmt.h"

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ void put3(char *line, int &len, float4 v, bool space) {
    if (space) line[len++] = ' ';
    len += gfmt::format_g(v.x, line + len);
    line[len++] = ' ';
    len += gfmt::format_g(v.y, line + len);
    line[len++] = ' ';
    len += gfmt::format_g(v.z, line + len);
}

__global__ void k_frame_lines(int n, int flags, const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                              const float *__restrict__ rho, const int *__restrict__ slot, float mass,
                              char *__restrict__ lines, unsigned *__restrict__ lens) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const int s = slot[id];
    char *line = lines + (size_t)id * kFrameLineCap;
    int len = 0;
    line[len++] = '\t';
    line[len++] = '\t';
    bool space = false;
    if (flags & kFramePosition) {
        put3(line, len, pos[s], space);
        space = true;
    }
    if (flags & kFrameVelocity) {
        put3(line, len, vel[s], space);
        space = true;
    }
    if (flags & kFrameDensity) {
        if (space) line[len++] = ' ';
        len += gfmt::format_g(rho[s], line + len);
        space = true;
    }
    if (flags & kFrameMass) {
        if (space) line[len++] = ' ';
        len += gfmt::format_g(mass, line + len);
    }
    line[len++] = '\n';
    lens[id] = (unsigned)len;
}

__global__ void k_frame_pack(int n, const char *__restrict__ lines, const unsigned *__restrict__ offset,
                             const unsigned *__restrict__ lens, char *__restrict__ out) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const char *src = lines + (size_t)id * kFrameLineCap;
    char *dst = out + offset[id];
    const unsigned len = lens[id];
    for (unsigned k = 0; k < len; k++) dst[k] = src[k];
}

void launch_frame_lines(int n, int flags, const float4 *pos, const float4 *vel, const float *rho,
                        const int *slot, float mass, FrameBufs &F, cudaStream_t s) {
    k_frame_lines<<<blocks_for(n, 128), 128, 0, s>>>(n, flags, pos, vel, rho, slot, mass, F.lines, F.lens);
    // the scan consumes its input: keep the lengths for the packing pass
    cudaMemcpyAsync(F.scan_in, F.lens, sizeof(unsigned) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    launch_cell_scan(F.scan_in, (unsigned)n, F.partials, F.offset, s);
    k_frame_pack<<<blocks_for(n, 128), 128, 0, s>>>(n, F.lines, F.offset, F.lens, F.out);
}

}  // namespace bbg
