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
// The triangulation table is derived on the host (cube faces walked around each region of
// corners at or below the iso value, ambiguous faces separating the smaller region, loops
// fanned from their first edge), not copied: vertices, normals and orientation are the
// reference's, triangles can differ where a case table choice does.
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

namespace {

// corners in the reference's data[] order (i, j, k offsets) and its 12 edges, each from
// its lower to its upper corner
constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}, {0, 1, 1}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6}, {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kMaxTri = 4;   // the derived table never needs more per cube

__constant__ signed char c_tri[256][3 * kMaxTri + 1];   // count, then edge triples
__constant__ int c_edge_dev[12][2];
__constant__ int c_corner_dev[8][3];

int edge_between(int a, int b) {
    for (int e = 0; e < 12; e++)
        if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
    return -1;
}

// The triangulation table: for each configuration (bit c set: corner c at or below iso),
// every face of the cube contributes directed segments between its crossing edges that keep
// the low corners on one side; the segments close into loops, fanned into triangles.
std::vector<signed char> derive_table() {
    // faces: 4 corners in counter-clockwise order seen from outside the cube
    std::vector<std::vector<int>> faces;
    for (int ax = 0; ax < 3; ax++) {
        for (int side = 0; side < 2; side++) {
            std::vector<int> cs;
            for (int c = 0; c < 8; c++)
                if (kCorner[c][ax] == side) cs.push_back(c);
            const int u = ax == 0 ? 1 : 0, v = ax == 2 ? 1 : 2;
            std::sort(cs.begin(), cs.end(), [&](int a, int b) {
                return std::atan2(kCorner[a][v] - 0.5, kCorner[a][u] - 0.5) <
                       std::atan2(kCorner[b][v] - 0.5, kCorner[b][u] - 0.5);
            });
            double p[3][3];
            for (int q = 0; q < 3; q++)
                for (int k = 0; k < 3; k++) p[q][k] = kCorner[cs[q]][k];
            const double e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
            const double e2[3] = {p[2][0] - p[1][0], p[2][1] - p[1][1], p[2][2] - p[1][2]};
            const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                  e1[0] * e2[1] - e1[1] * e2[0]};
            if (cr[ax] * (side ? 1.0 : -1.0) < 0) std::reverse(cs.begin(), cs.end());
            faces.push_back(cs);
        }
    }
    std::vector<signed char> table(256 * (3 * kMaxTri + 1), -1);
    for (int cfg = 0; cfg < 256; cfg++) {
        int low[8], nlow = 0;
        for (int c = 0; c < 8; c++) nlow += (low[c] = (cfg >> c) & 1);
        int next[12];
        for (int e = 0; e < 12; e++) next[e] = -1;
        for (const auto &f : faces) {
            int s = 0;
            for (int q = 0; q < 4; q++) s += low[f[q]];
            if (s == 0 || s == 4) continue;
            if (s == 2 && low[f[0]] == low[f[2]]) {
                // an ambiguous face: the smaller region's corners are cut off one by one
                const int target = nlow <= 4 ? 1 : 0;
                for (int q = 0; q < 4; q++) {
                    if (low[f[q]] != target) continue;
                    const int ein = edge_between(f[(q + 3) % 4], f[q]), eout = edge_between(f[q], f[(q + 1) % 4]);
                    if (target) next[ein] = eout;
                    else next[eout] = ein;
                }
            } else {
                int ein = -1, eout = -1;
                for (int q = 0; q < 4; q++) {
                    const int a = f[q], b = f[(q + 1) % 4];
                    if (!low[a] && low[b]) ein = edge_between(a, b);
                    if (low[a] && !low[b]) eout = edge_between(a, b);
                }
                next[ein] = eout;
            }
        }
        bool seen[12] = {};
        int ntri = 0;
        signed char *row = &table[(size_t)cfg * (3 * kMaxTri + 1)];
        for (int start = 0; start < 12; start++) {
            if (next[start] < 0 || seen[start]) continue;
            int loop[12], m = 0;
            for (int e = start; !seen[e]; e = next[e]) {
                seen[e] = true;
                loop[m++] = e;
            }
            for (int q = 1; q + 1 < m; q++) {
                row[1 + 3 * ntri] = (signed char)loop[0];
                row[2 + 3 * ntri] = (signed char)loop[q];
                row[3 + 3 * ntri] = (signed char)loop[q + 1];
                ntri++;
            }
        }
        row[0] = (signed char)ntri;
    }
    return table;
}

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
    ntri[id] = (unsigned)c_tri[cube_config(g, i, j, k)][0];
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
    const int nt = c_tri[cfg][0];
    unsigned t0 = tri_start[id];
    for (int t = 0; t < nt; t++) {
        int vid[3];
        for (int c = 0; c < 3; c++) {
            const int le = c_tri[cfg][1 + 3 * t + c];
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
    const std::vector<signed char> t = derive_table();
    cudaError_t e = cudaMemcpyToSymbol(c_tri, t.data(), t.size());
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
