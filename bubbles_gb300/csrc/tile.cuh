// tile.cuh -- tiles of the neighbour passes and the compact neighbour lists.
//
// Every neighbour pass runs one thread per particle in blocks of kTile consecutive slots
// of the cell-sorted arrays (a "tile").  The 27 neighbour cells of any particle in a tile
// lie, for each of the 9 (dy, dz) row offsets r, inside one contiguous range of linear
// cell ids, [first cell - 1 + off_r, last cell + 1 + off_r], i.e. one contiguous slot
// range starting at lo[r].  A neighbour j of a particle is therefore stored in 16 bits
// as (r << 12) | (j - lo[r]); every pass rebuilds the tile's 9 range starts from the
// grid (two loads per range) and decodes j = lo[r] + offset.
//
// Lists are chunk-major, 8 entries per 16-byte chunk: entry q of particle i is half-word
// q % 8 of list[(q / 8) * n + i], so a warp reads chunk c of 32 particles in one
// coalesced 512-byte load and a particle's usual 2-4 chunks are all requested before
// any neighbour is gathered.  A particle with more than kMaxList members, or with a
// member more than 4,095 slots into its range, is "wide" (kWide in its cell word) and
// re-tests its 27 cells exactly on every pass instead.
#pragma once

#include "bbg_internal.cuh"

namespace bbg {

constexpr int kTile = 128;          // slots per tile = threads per block of a neighbour pass
constexpr int kOffBits = 12;
constexpr int kOffLimit = 1 << kOffBits;

struct TileMap {
    int lo[9];      // first slot of range r
};

// The tile's 9 range starts from the grid (all threads of the block must call it).
__device__ __forceinline__ void tile_setup(const GridDev &g, const unsigned *__restrict__ cell,
                                           const unsigned *__restrict__ start, int n, TileMap &T) {
    if (threadIdx.x < 9) {
        const int s0 = blockIdx.x * kTile;
        const int r = threadIdx.x;
        const long long plane = (long long)g.nx * g.ny;
        const long long off = (long long)(r % 3 - 1) * g.nx + (long long)(r / 3 - 1) * plane;
        long long c0 = (long long)(__ldg(&cell[s0]) & ~kWide) - 1 + off;
        if (c0 < 0) c0 = 0;
        if (c0 > (long long)g.total) c0 = (long long)g.total;
        T.lo[r] = (int)__ldg(&start[c0]);
    }
    __syncthreads();
}

// The 9 row ranges of the 27 neighbour cells of cell c (reference neighbour list,
// src/core/grid.h:555-593) in z, y, x order: f(j, r) for every candidate slot j of range r.
template <class F>
__device__ __forceinline__ void tile_candidates(const GridDev &g, const unsigned *__restrict__ start,
                                                unsigned c, F &&f) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const unsigned plane = (unsigned)nx * (unsigned)ny;
    const int cz = (int)(c / plane);
    const unsigned rem = c - (unsigned)cz * plane;
    const int cy = (int)(rem / (unsigned)nx);
    const int cx = (int)(rem - (unsigned)cy * (unsigned)nx);
    const int x0 = cx > 0 ? cx - 1 : 0;
    const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
    const int z0 = cz > 0 ? cz - 1 : 0, z1 = cz + 1 < nz ? cz + 1 : nz - 1;
    const int y0 = cy > 0 ? cy - 1 : 0, y1 = cy + 1 < ny ? cy + 1 : ny - 1;
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            const int r = (z - cz + 1) * 3 + (y - cy + 1);
            const unsigned row = (unsigned)y * (unsigned)nx + (unsigned)z * plane;
            const unsigned b = __ldg(&start[row + (unsigned)x0]);
            const unsigned e = __ldg(&start[row + (unsigned)x1 + 1u]);
            for (unsigned j = b; j < e; ++j) f(j, r);
        }
    }
}

// Same visit order, for the density pass: f(j, base) with the list entry of j equal to
// j + base; *fits turns false when a range reaches past the 12-bit offset limit.
template <class F>
__device__ __forceinline__ void tile_candidates_coded(const GridDev &g, const unsigned *__restrict__ start,
                                                      const TileMap &T, unsigned c, bool *fits, F &&f) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const unsigned plane = (unsigned)nx * (unsigned)ny;
    const int cz = (int)(c / plane);
    const unsigned rem = c - (unsigned)cz * plane;
    const int cy = (int)(rem / (unsigned)nx);
    const int cx = (int)(rem - (unsigned)cy * (unsigned)nx);
    const int x0 = cx > 0 ? cx - 1 : 0;
    const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
    const int z0 = cz > 0 ? cz - 1 : 0, z1 = cz + 1 < nz ? cz + 1 : nz - 1;
    const int y0 = cy > 0 ? cy - 1 : 0, y1 = cy + 1 < ny ? cy + 1 : ny - 1;
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            const int r = (z - cz + 1) * 3 + (y - cy + 1);
            const unsigned lo = (unsigned)T.lo[r];
            const unsigned base = ((unsigned)r << kOffBits) - lo;
            const unsigned row = (unsigned)y * (unsigned)nx + (unsigned)z * plane;
            const unsigned b = __ldg(&start[row + (unsigned)x0]);
            const unsigned e = __ldg(&start[row + (unsigned)x1 + 1u]);
            if (e - lo > (unsigned)kOffLimit) *fits = false;
            for (unsigned j = b; j < e; ++j) f(j, base);
        }
    }
}

__device__ __forceinline__ unsigned list_slot(const TileMap &T, unsigned e) {
    return (unsigned)T.lo[e >> kOffBits] + (e & (kOffLimit - 1));
}

// Builds a particle's list in registers and stores each full chunk with one 16-byte
// store (a warp writes 512 contiguous bytes per chunk).
struct ChunkWriter {
    unsigned long long a = 0ull, b = 0ull;   // entries 0-3 and 4-7 of the open chunk
    int count = 0;                           // entries pushed (stores stop at kMaxList)
    __device__ __forceinline__ void store(uint4 *list, size_t n, unsigned i, int chunk) {
        list[(size_t)chunk * n + i] = make_uint4((unsigned)a, (unsigned)(a >> 32), (unsigned)b,
                                                 (unsigned)(b >> 32));
        a = b = 0ull;
    }
    __device__ __forceinline__ void push(uint4 *list, size_t n, unsigned i, unsigned e) {
        const int p = count & 7;
        const unsigned long long v = (unsigned long long)e << ((p & 3) * 16);
        if (p < 4) a |= v;
        else b |= v;
        if (p == 7 && count < kMaxList) store(list, n, i, count >> 3);
        count++;
    }
    __device__ __forceinline__ void finish(uint4 *list, size_t n, unsigned i) {
        if ((count & 7) != 0 && count < kMaxList) store(list, n, i, count >> 3);
    }
};

template <class F>
__device__ __forceinline__ void list_chunk(const TileMap &T, uint4 w, int m, F &f) {
    f(list_slot(T, w.x & 0xffffu));
    if (m > 1) f(list_slot(T, w.x >> 16));
    if (m > 2) f(list_slot(T, w.y & 0xffffu));
    if (m > 3) f(list_slot(T, w.y >> 16));
    if (m > 4) f(list_slot(T, w.z & 0xffffu));
    if (m > 5) f(list_slot(T, w.z >> 16));
    if (m > 6) f(list_slot(T, w.w & 0xffffu));
    if (m > 7) f(list_slot(T, w.w >> 16));
}

// f(j) for every member j != i of particle i's step-start neighbour set; wide particles
// re-test their candidates with the exact membership test at the step-start positions.
template <class F>
__device__ __forceinline__ void tile_members(const Params &P, const unsigned *__restrict__ start,
                                             const TileMap &T, const uint4 *__restrict__ list,
                                             const int *__restrict__ nbr, const float4 *__restrict__ pos0,
                                             unsigned cellw, int i, F &&f) {
    if (cellw & kWide) {
        const float4 pi = __ldg(&pos0[i]);
        tile_candidates(P.g, start, cellw & ~kWide, [&](unsigned j, int) {
            if (j == (unsigned)i) return;
            const float4 pj = __ldg(&pos0[j]);
            if (std_member(P, pi, pj, dist2(pi, pj))) f(j);
        });
        return;
    }
    const int cnt = __ldg(&nbr[i]) - 1;   // members other than i
    const size_t n = (size_t)P.n;
    const uint4 *l = list + i;
    // request the first four chunks (32 members) before gathering any neighbour
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    const uint4 w0 = cnt > 0 ? __ldg(l) : z;
    const uint4 w1 = cnt > 8 ? __ldg(l + n) : z;
    const uint4 w2 = cnt > 16 ? __ldg(l + 2 * n) : z;
    const uint4 w3 = cnt > 24 ? __ldg(l + 3 * n) : z;
    if (cnt > 0) list_chunk(T, w0, cnt, f);
    if (cnt > 8) list_chunk(T, w1, cnt - 8, f);
    if (cnt > 16) list_chunk(T, w2, cnt - 16, f);
    if (cnt > 24) list_chunk(T, w3, cnt - 24, f);
    for (int q = 32; q < cnt; q += 8) list_chunk(T, __ldg(l + (size_t)(q >> 3) * n), cnt - q, f);
}

}  // namespace bbg
