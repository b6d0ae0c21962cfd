// sdf.cu -- GenerateShapeSDF (src/core/shape.cpp:479-510) of an analytic shape on the device.
//
// One thread per grid node: the node's position (GetDataPosition of a vertex-centred
// FieldGrid3f), the shape's closest distance and IsInside, and the signed value
// max(|d|, 0.00001) with the inside sign (SetNodeSDFKernel, :409-424).
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__global__ void k_sdf_generate(ShapeDev shape, SdfDev g, float iz, float iz6, float *__restrict__ out) {
    const unsigned total = (unsigned)g.nx * (unsigned)g.ny * (unsigned)g.nz;
    const unsigned id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= total) return;
    // DimensionalIndex (src/core/grid.h:162-179)
    const unsigned plane = (unsigned)g.nx * (unsigned)g.ny;
    const unsigned k = id / plane, rem = id - k * plane;
    const unsigned j = rem / (unsigned)g.nx, i = rem % (unsigned)g.nx;
    const v3 p = V(fa(g.org[0], fm(g.sp[0], (float)i)), fa(g.org[1], fm(g.sp[1], (float)j)),
                   fa(g.org[2], fm(g.sp[2], (float)k)));
    const float d = shape_closest_point(shape, p, iz, iz6).sd;
    const bool interior = (shape.reverse != 0) == !(d < 0.f);
    const float psd = rmax(fabsf(d), 0.00001f);
    out[id] = interior ? -psd : psd;
}

void launch_sdf_generate(const ShapeDev &shape, const SdfDev &g, float iz, float iz6, float *out, cudaStream_t s) {
    const long long total = (long long)g.nx * g.ny * g.nz;
    k_sdf_generate<<<blocks_for(total, 256), 256, 0, s>>>(shape, g, iz, iz6, out);
}

// Shape queries at n points of collider `shape`: the field's Sample and Gradient (when it
// has one), Shape::ClosestPoint and IsInside as the collision code evaluates them.
__global__ void k_shape_query(Params P, int index, int n, const float *__restrict__ pts, float *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const ShapeDev &s = P.shapes[index];
    const v3 p = V(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
    float *o = out + 14 * (size_t)q;   // sample, gradient xyz, point xyz, normal xyz, distance, inside, 2 spare
    Cpq c;
    bool inside;
    float sample = 0.f;
    v3 grad = V(0.f, 0.f, 0.f);
    if (s.sdf >= 0) {
        const SdfDev &g = P.sdf[s.sdf];
        sample = sdf_sample(g, p);
        grad = sdf_gradient(g, p);
        c = sdf_closest_point(s, g, p);
        inside = sample < 0.f;
    } else {
        c = shape_closest_point(s, p, P.iz, P.iz6);
        inside = (s.reverse != 0) == !(c.sd < 0.f);
    }
    o[0] = sample;
    o[1] = grad.x; o[2] = grad.y; o[3] = grad.z;
    o[4] = c.point.x; o[5] = c.point.y; o[6] = c.point.z;
    o[7] = c.normal.x; o[8] = c.normal.y; o[9] = c.normal.z;
    o[10] = c.sd;
    o[11] = inside ? 1.f : 0.f;
    o[12] = 0.f;
    o[13] = 0.f;
}

void launch_shape_query(const Params &P, int index, int n, const float *pts, float *out, cudaStream_t s) {
    k_shape_query<<<blocks_for(n, 128), 128, 0, s>>>(P, index, n, pts, out);
}

}  // namespace bbg
