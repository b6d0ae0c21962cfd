// mc.cu -- marching cubes of a vertex-centred field on the device (MarchingCubes,
// src/reconstruction/marching_cubes.cpp:204-457).
//
// The reference keeps the cubes whose corners straddle the iso value, places a vertex on
// each crossing edge at the linear zero of (value - iso) with the reference's clamped
// weight, interpolates the corners' central-difference gradients for its normal, and
// joins the vertices with its case table, deduplicating them by edge.  Here:
// - one thread per cube classifies it and counts its triangles;
// - one thread per grid edge (x, y and z edges) flags the crossing ones; a scan numbers
//   them, so each vertex is made once, in the same float operations as the reference
//   (every edge runs from its lower to its upper node, so the position does not depend on
//   which cube computes it);
// - one thread per cube writes its triangles.
// The triangles follow the reference's case table (marching_cubes_table.h,
// triangleConnectionTable3D): triangles are only identical when every case is
// triangulated the same way, so that table's content is kept, re-encoded below as one
// packed 64-bit word per case.
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

#include <cstring>

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

namespace {

// corners in the reference's data[] order (i, j, k offsets) and its 12 edges, each from
// its lower to its upper corner
constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6}, {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// The case table: for configuration c (bit q set: corner q at or below the iso value),
// bits 60..63 of kCase[c] hold its triangle count and bits 4m..4m+3 the m-th edge of its
// triangles, three per triangle in the reference's winding.
constexpr unsigned long long kCase[256] = {
    0x0000000000000000ull, 0x1000000000000380ull, 0x1000000000000910ull, 0x2000000000189381ull,
    0x1000000000000a21ull, 0x2000000000a21380ull, 0x2000000000920a29ull, 0x300000089a8a2382ull,
    0x10000000000002b3ull, 0x20000000000b82b0ull, 0x2000000000b32091ull, 0x3000000b89b912b1ull,
    0x20000000003ab1a3ull, 0x3000000ab8a801a0ull, 0x30000009ab9b3093ull, 0x2000000000b8aa89ull,
    0x1000000000000874ull, 0x2000000000437034ull, 0x2000000000748910ull, 0x3000000137174914ull,
    0x2000000000748a21ull, 0x3000000a21403743ull, 0x3000000748209a29ull, 0x40004973727929a2ull,
    0x20000000002b3748ull, 0x300000040242b74bull, 0x3000000b32748109ull, 0x40001292b9b49b74ull,
    0x3000000487ab31a3ull, 0x40004b7401b41ab1ull, 0x400030bab9b09874ull, 0x3000000ab99b4b74ull,
    0x1000000000000459ull, 0x2000000000380459ull, 0x2000000000051450ull, 0x3000000513538458ull,
    0x2000000000459a21ull, 0x3000000594a21803ull, 0x3000000204245a25ull, 0x40008434535235a2ull,
    0x2000000000b32459ull, 0x3000000594b802b0ull, 0x3000000b32510450ull, 0x4000584b82852512ull,
    0x300000045931ab3aull, 0x4000ab81a8180594ull, 0x400030bab5b05045ull, 0x3000000b8aa85845ull,
    0x2000000000975879ull, 0x3000000375359039ull, 0x3000000751710870ull, 0x2000000000753351ull,
    0x300000021a759879ull, 0x400037503505921aull, 0x400025a758528208ull, 0x30000007533525a2ull,
    0x30000002b3987597ull, 0x4000b72029279759ull, 0x4000751871810b32ull, 0x300000051771b12bull,
    0x4000b3a31a758859ull, 0x50aba010b7905075ull, 0x507570805a30b0abull, 0x20000000005b75abull,
    0x100000000000056aull, 0x20000000006a5380ull, 0x20000000006a5109ull, 0x30000006a5891381ull,
    0x2000000000162561ull, 0x3000000803621561ull, 0x3000000620609569ull, 0x4000823625285895ull,
    0x200000000056ab32ull, 0x300000056a02b80bull, 0x30000006a5b32910ull, 0x4000b892b92916a5ull,
    0x3000000315356b36ull, 0x40006b51505b0b80ull, 0x40009505606306b3ull, 0x300000089bb96956ull,
    0x20000000008746a5ull, 0x3000000a56374034ull, 0x30000007486a5091ull, 0x400049737179156aull,
    0x3000000874156216ull, 0x4000743403625521ull, 0x4000620560509748ull, 0x5962695923497937ull,
    0x300000056a4872b3ull, 0x4000b720242746a5ull, 0x40006a5b32874910ull, 0x56a54b7b492b9129ull,
    0x40006b51535b3748ull, 0x5b404b7b016b5b15ull, 0x574836b630560950ull, 0x40009b7974b96956ull,
    0x2000000000a4694aull, 0x3000000380a946a4ull, 0x300000004606a10aull, 0x4000a16468618138ull,
    0x3000000462421941ull, 0x4000462942921803ull, 0x2000000000624420ull, 0x3000000624428238ull,
    0x300000032b46a94aull, 0x40006a4a94b82280ull, 0x4000a164606102b3ull, 0x51b8b12184a16146ull,
    0x400036b319639469ull, 0x514641916b0181b8ull, 0x30000004600636b3ull, 0x200000000086b846ull,
    0x3000000a98a876a7ull, 0x4000a76a907a0370ull, 0x40000818717a176aull, 0x300000037117a76aull,
    0x4000768981861621ull, 0x5937390976192962ull, 0x3000000206607087ull, 0x2000000000276237ull,
    0x400076898a86ab32ull, 0x57a9a76790b72702ull, 0x5b32a767a1871081ull, 0x400017616a71b12bull,
    0x563136b619768698ull, 0x200000000076b190ull, 0x400006b0b3607087ull, 0x10000000000006b7ull,
    0x1000000000000b67ull, 0x200000000067b803ull, 0x200000000067b910ull, 0x300000067b138918ull,
    0x20000000007b621aull, 0x30000007b6803a21ull, 0x30000007b69a2092ull, 0x400089a38a3a27b6ull,
    0x2000000000726327ull, 0x3000000026067807ull, 0x3000000910732672ull, 0x4000678891681261ull,
    0x300000073171a67aull, 0x4000801781a7167aull, 0x40007a69a0a70730ull, 0x30000009a88a7a67ull,
    0x200000000068b486ull, 0x3000000640603b63ull, 0x3000000109648b68ull, 0x400063b139369649ull,
    0x30000001a28b6486ull, 0x4000640b60b03a21ull, 0x40009a2920b648b4ull, 0x536463b34923a39aull,
    0x3000000264248328ull, 0x2000000000264240ull, 0x4000834642432091ull, 0x3000000642241491ull,
    0x40001a6648168318ull, 0x300000040660a01aull, 0x539a9303a6834364ull, 0x20000000004a649aull,
    0x2000000000b67594ull, 0x300000067b594380ull, 0x3000000b67045105ull, 0x400051345343867bull,
    0x3000000b6721a459ull, 0x4000594380a217b6ull, 0x4000204a24a45b67ull, 0x567b25a523453843ull,
    0x3000000945267327ull, 0x4000786260680459ull, 0x4000045051673263ull, 0x5851584812786826ull,
    0x400073167161a459ull, 0x5459078701671a61ull, 0x5a737a6a305a4a04ull, 0x4000a84a458a7a67ull,
    0x300000098b9b6596ull, 0x4000590650360b63ull, 0x4000b65510b508b0ull, 0x30000001355363b6ull,
    0x400065b8b9b59a21ull, 0x5a21965690b603b0ull, 0x552025a50865b58bull, 0x400035a3a2536b63ull,
    0x4000283265825985ull, 0x3000000260069659ull, 0x5826283865081851ull, 0x2000000000612651ull,
    0x5698965683a61631ull, 0x400006505960a01aull, 0x2000000000a65830ull, 0x100000000000065aull,
    0x2000000000b57a5bull, 0x300000003857ba5bull, 0x3000000091ba57b5ull, 0x40001381897ba57aull,
    0x300000015717b21bull, 0x4000b27571721380ull, 0x40007b2209729579ull, 0x5289823295b27257ull,
    0x3000000573532a52ull, 0x400052a578258028ull, 0x40002a37353a5109ull, 0x525752a278129289ull,
    0x2000000000573531ull, 0x3000000571170780ull, 0x3000000735539309ull, 0x2000000000795789ull,
    0x30000008ba8a5485ull, 0x400003bba50b5405ull, 0x400054aba8a48910ull, 0x541314943b54a4baull,
    0x40008548b2582152ull, 0x5b151b2b543b0b40ull, 0x558b8545b2950520ull, 0x20000000003b2549ull,
    0x4000483543253a52ull, 0x30000000244252a5ull, 0x5910854583a532a3ull, 0x40002492914252a5ull,
    0x3000000153358548ull, 0x2000000000501540ull, 0x4000530509358548ull, 0x1000000000000549ull,
    0x3000000ba9b947b4ull, 0x4000ba97b9794380ull, 0x4000b470414b1ba1ull, 0x54bab474a1843413ull,
    0x4000219b294b97b4ull, 0x53801b2b197b9479ull, 0x300000004224b47bull, 0x400042343824b47bull,
    0x4000947732972a92ull, 0x570207872a4797a9ull, 0x5a040a1a472a3a73ull, 0x20000000004782a1ull,
    0x3000000317714194ull, 0x4000178180714194ull, 0x2000000000347304ull, 0x1000000000000784ull,
    0x20000000008ba8a9ull, 0x3000000a9bb93903ull, 0x3000000ba88a0a10ull, 0x2000000000a3ba13ull,
    0x30000008b99b1b21ull, 0x40009b2921b93903ull, 0x2000000000b08b20ull, 0x1000000000000b23ull,
    0x300000098aa82832ull, 0x20000000002902a9ull, 0x40008a1810a82832ull, 0x10000000000002a1ull,
    0x2000000000819831ull, 0x1000000000000190ull, 0x1000000000000830ull, 0x0000000000000000ull
};

__constant__ unsigned long long c_case[256];
__constant__ int c_edge_dev[12][2];
__constant__ int c_corner_dev[8][3];

__device__ __forceinline__ int case_triangles(int cfg) { return (int)(c_case[cfg] >> 60); }
__device__ __forceinline__ int case_edge(int cfg, int m) { return (int)((c_case[cfg] >> (4 * m)) & 15ull); }

struct McGrid {
    const float *v;
    int nx, ny, nz;
    float org[3], sp[3];
    float inv[3];   // (float)(1.0 / spacing)
    float iso;
};

__device__ __forceinline__ float node_value(const McGrid &g, int i, int j, int k) {
    return __ldg(&g.v[(unsigned)i + (unsigned)j * g.nx + (unsigned)k * (unsigned)g.nx * g.ny]);
}

__device__ __forceinline__ int cube_config(const McGrid &g, int i, int j, int k) {
    int cfg = 0;
    for (int c = 0; c < 8; c++)
        if (node_value(g, i + c_corner_dev[c][0], j + c_corner_dev[c][1], k + c_corner_dev[c][2]) <= g.iso)
            cfg |= 1 << c;
    return cfg;
}

// cube index with x slowest and z fastest, the reference's cubeId order
__device__ __forceinline__ void cube_of(const McGrid &g, long long id, int &i, int &j, int &k) {
    const long long zl = g.nz - 1, yl = g.ny - 1;
    k = (int)(id % zl);
    j = (int)((id / zl) % yl);
    i = (int)(id / (yl * zl));
}

__global__ void k_mc_cubes(McGrid g, long long cubes, unsigned *__restrict__ ntri) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= cubes) return;
    int i, j, k;
    cube_of(g, id, i, j, k);
    ntri[id] = (unsigned)case_triangles(cube_config(g, i, j, k));
}

// edge e = axis * nodes + node: the edge from node (i, j, k) along the axis
__global__ void k_mc_edges(McGrid g, long long nodes, unsigned *__restrict__ crossing) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * nodes) return;
    const int axis = (int)(e / nodes);
    const long long n = e - axis * nodes;
    const int i = (int)(n % g.nx), j = (int)((n / g.nx) % g.ny), k = (int)(n / ((long long)g.nx * g.ny));
    const int i1 = i + (axis == 0), j1 = j + (axis == 1), k1 = k + (axis == 2);
    unsigned c = 0;
    if (i1 < g.nx && j1 < g.ny && k1 < g.nz)
        c = ((node_value(g, i, j, k) <= g.iso) != (node_value(g, i1, j1, k1) <= g.iso)) ? 1u : 0u;
    crossing[e] = c;
}

// grad (marching_cubes.cpp:121-159): central differences, one-sided at the first node and
// repeated at the last, all scaled by 0.5 / spacing
__device__ v3 node_gradient(const McGrid &g, int i, int j, int k) {
    int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1, kp = k + 1, km = k - 1;
    if (i > g.nx - 2) ip = i;
    else if (i == 0) im = 0;
    if (j > g.ny - 2) jp = j;
    else if (j == 0) jm = 0;
    if (k > g.nz - 2) kp = k;
    else if (k == 0) km = 0;
    return V(fm(fm(0.5f, g.inv[0]), fs(node_value(g, ip, j, k), node_value(g, im, j, k))),
             fm(fm(0.5f, g.inv[1]), fs(node_value(g, i, jp, k), node_value(g, i, jm, k))),
             fm(fm(0.5f, g.inv[2]), fs(node_value(g, i, j, kp), node_value(g, i, j, km))));
}

__device__ __forceinline__ v3 node_position(const McGrid &g, int i, int j, int k) {
    return V(fa(g.org[0], fm(g.sp[0], (float)i)), fa(g.org[1], fm(g.sp[1], (float)j)), fa(g.org[2], fm(g.sp[2], (float)k)));
}

// Lerp(p0, p1, a) = (1 - a) p0 + a p1
__device__ __forceinline__ v3 vlerp(v3 p0, v3 p1, float a) { return vadd(vmul(p0, fs(1.f, a)), vmul(p1, a)); }

__global__ void k_mc_vertices(McGrid g, long long nodes, const unsigned *__restrict__ crossing,
                              const unsigned *__restrict__ index, float *__restrict__ points,
                              float *__restrict__ normals) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3 * nodes || !crossing[e]) return;
    const int axis = (int)(e / nodes);
    const long long n = e - axis * nodes;
    const int i = (int)(n % g.nx), j = (int)((n / g.nx) % g.ny), k = (int)(n / ((long long)g.nx * g.ny));
    const int i1 = i + (axis == 0), j1 = j + (axis == 1), k1 = k + (axis == 2);
    // distanceToZeroLevelSet, clamped to [1e-6, 0.999999]
    const float phi0 = fs(node_value(g, i, j, k), g.iso), phi1 = fs(node_value(g, i1, j1, k1), g.iso);
    const float s = fa(fabsf(phi0), fabsf(phi1));
    float a = s > 0.0001f ? fdv(fabsf(phi0), s) : 0.5f;
    if ((double)a < 0.000001) a = 0.000001f;
    if ((double)a > 0.999999) a = 0.999999f;
    const v3 p = vlerp(node_position(g, i, j, k), node_position(g, i1, j1, k1), a);
    v3 nn = vlerp(node_gradient(g, i, j, k), node_gradient(g, i1, j1, k1), a);
    // safeNormalize
    const float l2 = vlen2(nn);
    if ((double)l2 > 0.0 && !((double)fabsf(l2) < 1e-8)) nn = vdiv(nn, vlen(nn));
    const unsigned q = index[e];
    points[3 * (size_t)q] = p.x;
    points[3 * (size_t)q + 1] = p.y;
    points[3 * (size_t)q + 2] = p.z;
    normals[3 * (size_t)q] = nn.x;
    normals[3 * (size_t)q + 1] = nn.y;
    normals[3 * (size_t)q + 2] = nn.z;
}

__global__ void k_mc_triangles(McGrid g, long long cubes, long long nodes, const unsigned *__restrict__ tri_start,
                               const unsigned *__restrict__ vindex, int rotate, int *__restrict__ tris) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= cubes) return;
    int i, j, k;
    cube_of(g, id, i, j, k);
    const int cfg = cube_config(g, i, j, k);
    const int nt = case_triangles(cfg);
    unsigned t0 = tri_start[id];
    for (int t = 0; t < nt; t++) {
        int vid[3];
        for (int c = 0; c < 3; c++) {
            const int le = case_edge(cfg, 3 * t + c);
            const int a = c_edge_dev[le][0], b = c_edge_dev[le][1];
            const int ai = i + c_corner_dev[a][0], aj = j + c_corner_dev[a][1], ak = k + c_corner_dev[a][2];
            const int axis = c_corner_dev[b][0] != c_corner_dev[a][0] ? 0 : (c_corner_dev[b][1] != c_corner_dev[a][1] ? 1 : 2);
            const long long node = (long long)ai + (long long)aj * g.nx + (long long)ak * g.nx * g.ny;
            vid[c] = (int)vindex[axis * nodes + node];
        }
        int *o = tris + 3 * (size_t)(t0 + t);
        o[0] = vid[0];
        o[1] = rotate ? vid[2] : vid[1];
        o[2] = rotate ? vid[1] : vid[2];
    }
}

bool tables_ready = false;

}  // namespace

cudaError_t mc_prepare() {
    if (tables_ready) return cudaSuccess;
    cudaError_t e = cudaMemcpyToSymbol(c_case, kCase, sizeof(kCase));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_edge_dev, kEdge, sizeof(kEdge));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_corner_dev, kCorner, sizeof(kCorner));
    if (e == cudaSuccess) tables_ready = true;
    return e;
}

// Counts: returns the triangles and crossing edges (vertices) of the field (synchronises).
cudaError_t mc_count(const McInput &in, unsigned *ntri_cube, unsigned *tri_start, unsigned *tri_part,
                     unsigned *crossing, unsigned *flag_copy, unsigned *vindex, unsigned *v_part, unsigned *h,
                     size_t *ntri, size_t *nvert, cudaStream_t s) {
    McGrid g;
    g.v = in.values;
    g.nx = in.nodes[0];
    g.ny = in.nodes[1];
    g.nz = in.nodes[2];
    for (int k = 0; k < 3; k++) {
        g.org[k] = in.origin[k];
        g.sp[k] = in.spacing[k];
        g.inv[k] = in.inv[k];
    }
    g.iso = in.iso;
    const long long cubes = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
    const long long nodes = (long long)g.nx * g.ny * g.nz;
    k_mc_cubes<<<blocks_for(cubes, 256), 256, 0, s>>>(g, cubes, ntri_cube);
    launch_cell_scan(ntri_cube, (unsigned)cubes, tri_part, tri_start, s);
    k_mc_edges<<<blocks_for(3 * nodes, 256), 256, 0, s>>>(g, nodes, crossing);
    // the scan zeroes its input: keep the crossing flags, scan a copy
    cudaMemcpyAsync(flag_copy, crossing, sizeof(unsigned) * (size_t)(3 * nodes), cudaMemcpyDeviceToDevice, s);
    launch_cell_scan(flag_copy, (unsigned)(3 * nodes), v_part, vindex, s);
    cudaMemcpyAsync(h, tri_start + cubes, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(h + 1, vindex + 3 * nodes, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    *ntri = h[0];
    *nvert = h[1];
    return e;
}

void mc_emit(const McInput &in, const unsigned *tri_start, const unsigned *crossing, const unsigned *vindex,
             int rotate, float *points, float *normals, int *tris, cudaStream_t s) {
    McGrid g;
    g.v = in.values;
    g.nx = in.nodes[0];
    g.ny = in.nodes[1];
    g.nz = in.nodes[2];
    for (int k = 0; k < 3; k++) {
        g.org[k] = in.origin[k];
        g.sp[k] = in.spacing[k];
        g.inv[k] = in.inv[k];
    }
    g.iso = in.iso;
    const long long cubes = (long long)(g.nx - 1) * (g.ny - 1) * (g.nz - 1);
    const long long nodes = (long long)g.nx * g.ny * g.nz;
    k_mc_vertices<<<blocks_for(3 * nodes, 256), 256, 0, s>>>(g, nodes, crossing, vindex, points, normals);
    k_mc_triangles<<<blocks_for(cubes, 256), 256, 0, s>>>(g, cubes, nodes, tri_start, vindex, rotate, tris);
}

}  // namespace bbg
