// boundary.cu -- LNM boundary classification (src/boundaries/lnm.h:24-139, 245-275, the
// fast variant) on the sorted grid.
//
// The reference walks its cells' chains; here a cell's particles are the slot range of the
// last grid distribution.  One thread per cell: L1 when the cell holds particles and lies on
// the grid's border (fewer than 27 neighbour cells) or next to an empty cell; then L2 when
// it holds particles, is not L1 and has an L1 neighbour holding at most delta particles.
// One thread per particle then writes its cell's level in the caller's order.
#include "bbg_internal.cuh"
#include "bbg_kernels.h"

namespace bbg {

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

namespace {

__device__ __forceinline__ unsigned held(const unsigned *start, unsigned c) { return start[c + 1] - start[c]; }

__global__ void k_lnm_l1(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    level[c] = -1;
    if (held(start, c) < 1) return;
    const int x = (int)(c % (unsigned)g.nx), y = (int)((c / (unsigned)g.nx) % (unsigned)g.ny);
    const int z = (int)(c / ((unsigned)g.nx * (unsigned)g.ny));
    const int x0 = x > 0 ? x - 1 : 0, x1 = x + 1 < g.nx ? x + 1 : g.nx - 1;
    const int y0 = y > 0 ? y - 1 : 0, y1 = y + 1 < g.ny ? y + 1 : g.ny - 1;
    const int z0 = z > 0 ? z - 1 : 0, z1 = z + 1 < g.nz ? z + 1 : g.nz - 1;
    if ((x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1) != 27) {   // GetNeighborsOf count
        level[c] = 1;
        return;
    }
    for (int k = z0; k <= z1; k++)
        for (int j = y0; j <= y1; j++)
            for (int i = x0; i <= x1; i++)
                if (held(start, (unsigned)i + (unsigned)j * g.nx + (unsigned)k * g.nx * g.ny) == 0) {
                    level[c] = 1;
                    return;
                }
}

__global__ void k_lnm_l2(GridDev g, const unsigned *__restrict__ start, int *__restrict__ level, int delta) {
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.total) return;
    if (held(start, c) < 1 || level[c] == 1) return;
    const int x = (int)(c % (unsigned)g.nx), y = (int)((c / (unsigned)g.nx) % (unsigned)g.ny);
    const int z = (int)(c / ((unsigned)g.nx * (unsigned)g.ny));
    for (int k = z > 0 ? z - 1 : 0; k <= (z + 1 < g.nz ? z + 1 : g.nz - 1); k++)
        for (int j = y > 0 ? y - 1 : 0; j <= (y + 1 < g.ny ? y + 1 : g.ny - 1); j++)
            for (int i = x > 0 ? x - 1 : 0; i <= (x + 1 < g.nx ? x + 1 : g.nx - 1); i++) {
                const unsigned nb = (unsigned)i + (unsigned)j * g.nx + (unsigned)k * g.nx * g.ny;
                // an L2 write never turns a cell into or out of L1, so the reads are stable
                if (level[nb] == 1 && held(start, nb) <= (unsigned)delta) {
                    level[c] = 2;
                    return;
                }
            }
}

__global__ void k_lnm_particles(int n, const unsigned *__restrict__ cell, const int *__restrict__ pid,
                                const int *__restrict__ level, int *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int L = level[cell[q] & ~kWide];
    out[pid[q]] = (L == 1 || L == 2) ? L : 0;
}

}  // namespace

void launch_lnm(const GridDev &g, const unsigned *start, const unsigned *cell, const int *pid, int n, int delta,
                int *level, int *out, cudaStream_t s) {
    k_lnm_l1<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level);
    k_lnm_l2<<<blocks_for(g.total, 256), 256, 0, s>>>(g, start, level, delta);
    k_lnm_particles<<<blocks_for(n, 256), 256, 0, s>>>(n, cell, pid, level, out);
}

}  // namespace bbg
