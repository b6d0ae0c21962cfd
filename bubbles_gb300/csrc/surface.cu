// surface.cu -- the surface app's particle-to-field step (apps/surface.cpp:276-470,
// ParticlesToSDF_Surface with ZhuBridsonSDF or SphSDF) on the sorted grid.
//
// One thread per node of the vertex-centred field: the node's position, the domain test,
// the hashed cell and its 27 neighbours in the reference's order (y, then x, then z), each
// cell's particles in chain order (the slot range of the last distribution).  Every float
// operation is explicitly rounded in the reference's order; the steps the reference takes
// in double (the cubic weight of Zhu-Bridson, the std kernel's constant) are double here.
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

namespace bbg {

namespace {

__device__ __forceinline__ float dist3(v3 a, float4 b) {
    const float ex = fs(a.x, b.x), ey = fs(a.y, b.y), ez = fs(a.z, b.z);
    return __fsqrt_rn(fa(fa(fm(ex, ex), fm(ey, ey)), fm(ez, ez)));
}

__global__ void k_particle_sdf(SurfaceArgs A, float *__restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)A.nodes[0] * A.nodes[1] * A.nodes[2];
    if (i >= total) return;
    // DimensionalIndex and FieldGrid3f::GetDataPosition (vertex centred)
    const unsigned ux = (unsigned)(i % A.nodes[0]);
    const unsigned uy = (unsigned)((i / A.nodes[0]) % A.nodes[1]);
    const unsigned uz = (unsigned)(i / ((long long)A.nodes[0] * A.nodes[1]));
    const v3 p = V(fa(A.org[0], fm(A.sp[0], (float)ux)), fa(A.org[1], fm(A.sp[1], (float)uy)),
                   fa(A.org[2], fm(A.sp[2], (float)uz)));
    const GridDev &g = A.g;
    if (!inside3(p, V(g.bmin[0], g.bmin[1], g.bmin[2]), V(g.bmax[0], g.bmax[1], g.bmax[2]), A.iz6)) {
        out[i] = A.inf;
        return;
    }
    unsigned bad = 0;
    const unsigned c = grid_hash(g, make_float4(p.x, p.y, p.z, 0.f), A.iz, &bad);
    const int cx = (int)(c % (unsigned)g.nx), cy = (int)((c / (unsigned)g.nx) % (unsigned)g.ny);
    const int cz = (int)(c / ((unsigned)g.nx * (unsigned)g.ny));
    const float R = A.radius;
    float wsum = 0.f, ax = 0.f, ay = 0.f, az = 0.f;
    for (int y = max(cy - 1, 0); y <= min(cy + 1, g.ny - 1); y++)
        for (int x = max(cx - 1, 0); x <= min(cx + 1, g.nx - 1); x++)
            for (int z = max(cz - 1, 0); z <= min(cz + 1, g.nz - 1); z++) {
                const unsigned nb = (unsigned)x + (unsigned)y * g.nx + (unsigned)z * g.nx * g.ny;
                for (unsigned s = A.start[nb]; s < A.start[nb + 1]; s++) {
                    const float4 xi = A.pos[s];
                    const float d = dist3(p, xi);
                    if (A.method == 0) {
                        // ZhuBridsonSDF: k_cub(|p - x| / R) = Max(0, (1 - s^2)^3), the cube in double
                        if (d < R) {
                            const float t = fdv(d, R);
                            const double q = __dsub_rn(1.0, (double)fm(t, t));
                            const float cub = __double2float_rn(__dmul_rn(__dmul_rn(q, q), q));
                            const float w = 0.f < cub ? cub : 0.f;
                            wsum = fa(wsum, w);
                            ax = fa(ax, fm(xi.x, w));
                            ay = fa(ay, fm(xi.y, w));
                            az = fa(az, fm(xi.z, w));
                        }
                    } else {
                        // SphSDF: (mass / rho) W_std(d) at radius R (kernel.cpp:123-132)
                        const float d2 = fm(d, d);
                        const float of = fs(d2, A.r2);
                        float w = 0.f;
                        if (!(fabsf(of) < A.iz || of > 0.f)) {
                            const double x = (double)fs(1.f, fdv(d2, A.r2));
                            w = __double2float_rn(__dmul_rn(__dmul_rn(__dmul_rn(A.wc, x), x), x));
                        }
                        wsum = fa(wsum, fm(fdv(A.mass, A.rho[s]), w));
                    }
                }
            }
    if (A.method != 0) {
        out[i] = fs(0.5f, wsum);
    } else if (wsum > 0.f) {
        const float inv = __double2float_rn(__ddiv_rn(1.0, (double)wsum));
        const float4 m = make_float4(fm(ax, inv), fm(ay, inv), fm(az, inv), 0.f);
        out[i] = fs(dist3(p, m), A.offset);
    } else {
        out[i] = A.inf;
    }
}

}  // namespace

void launch_particle_sdf(const SurfaceArgs &A, float *out, cudaStream_t s) {
    const long long total = (long long)A.nodes[0] * A.nodes[1] * A.nodes[2];
    k_particle_sdf<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(A, out);
}

}  // namespace bbg
