// tile.cuh -- tiles of the neighbour passes and the neighbour lists.
//
// Every neighbour pass runs one thread per particle in blocks of consecutive slots of the
// cell-sorted arrays (a "tile": the block size, 64 to 256, a tuning parameter).
//
// The density pass records each particle's neighbour set (the reference bucket) as a
// list, member-major: entry q of particle i is list[q * n + i], so entry q of 32
// particles is written and read with one coalesced access.  Later passes request several
// entries and then the neighbours' records before using any (tile_members).  A particle
// with more than kMaxList members is "wide" (kWide in its cell word) and re-tests its 27
// cells exactly on every pass instead.
//
// Entries are absolute slot indices (32 bit).  A build-time alternative
// (BBG_LIST_BITS=16) halves the list: the 27 neighbour cells of any particle in a tile
// lie, for each of the 9 (dy, dz) row offsets r, inside one contiguous slot range starting
// at lo[r] ([first cell - 1 + off_r, last cell + 1 + off_r] in linear cell ids), so j is
// stored as (r << 12) | (j - lo[r]) and every pass rebuilds the tile's 9 starts; on GB300
// the decoding cost more issue slots than the smaller list saved (13-16 % slower steps).
#pragma once

#include "bbg_internal.cuh"

namespace bbg {

constexpr int kTile = 128;          // default tile: slots per tile = threads per block
constexpr int kMaxTile = 256;       // largest block size a neighbour pass is launched with
#ifndef BBG_GATHER_BATCH
#define BBG_GATHER_BATCH 4
#endif
// members whose neighbour records are requested together (build-time tuning knob)
constexpr int kGatherBatch = BBG_GATHER_BATCH;
constexpr int kOffBits = 12;
constexpr int kOffLimit = 1 << kOffBits;

struct TileMap {
    int lo[9];      // first slot of range r
};

#ifndef BBG_LIST_BITS
#define BBG_LIST_BITS 32
#endif
#if BBG_LIST_BITS == 32
// absolute slot indices (4 bytes per member, no decoding): measured faster on GB300 than
// the 16-bit tile-relative entries, whose decoding costs issue slots in every pass
using ListEntry = unsigned;
__device__ __forceinline__ unsigned list_slot(const TileMap &, unsigned e) { return e; }
__device__ __forceinline__ unsigned list_code(unsigned j, unsigned) { return j; }
constexpr bool kListRelative = false;
#else
using ListEntry = unsigned short;
__device__ __forceinline__ unsigned list_slot(const TileMap &T, unsigned e) {
    return (unsigned)T.lo[e >> kOffBits] + (e & (kOffLimit - 1));
}
__device__ __forceinline__ unsigned short list_code(unsigned j, unsigned base) {
    return (unsigned short)(j + base);
}
constexpr bool kListRelative = true;
#endif

// The 9 range starts of the tile whose first slot is s0, from the grid (all threads of the
// block must call it; a no-op with absolute list entries).
__device__ __forceinline__ void tile_setup_at(const GridDev &g, const unsigned *__restrict__ cell,
                                              const unsigned *__restrict__ start, int s0, TileMap &T) {
    if (!kListRelative) return;
    __syncthreads();   // a previous tile of the same block may still read T
    if (threadIdx.x < 9) {
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

// Tile of block b among `tiles`.  With P.tile_sms = G > 0, blocks b, b + G, b + 2G, ... take
// consecutive tiles: tile = (b mod G) * per + b / G, per = ceil(tiles / G).  The block
// scheduler's first waves place those blocks on the same SM (one block per SM per round), so
// the blocks resident on an SM walk neighbouring tiles and share neighbour records in its L1.
// The grid is G * per blocks; a block whose tile is past the last one has no work.
__device__ __forceinline__ int tile_of_block(const Params &P, int b, int tiles) {
    const int G = P.tile_sms;
    if (G <= 0) return b;
    const int per = (tiles + G - 1) / G;
    return (b % G) * per + b / G;
}

// The range starts of the block's own tile (slots blockIdx.x * blockDim.x on).
__device__ __forceinline__ void tile_setup(const GridDev &g, const unsigned *__restrict__ cell,
                                           const unsigned *__restrict__ start, int n, TileMap &T) {
    (void)n;
    tile_setup_at(g, cell, start, blockIdx.x * blockDim.x, T);
}

// The 9 row ranges of the 27 neighbour cells of cell c in z, y, x order: f(r, b, e) for
// range r = slots [b, e).
template <class F>
__device__ __forceinline__ void tile_rows(const GridDev &g, const unsigned *__restrict__ start, unsigned c,
                                          F &&f) {
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
            const unsigned row = (unsigned)y * (unsigned)nx + (unsigned)z * plane;
            f((z - cz + 1) * 3 + (y - cy + 1), __ldg(&start[row + (unsigned)x0]),
              __ldg(&start[row + (unsigned)x1 + 1u]));
        }
    }
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

// The rows of tile_rows for the density pass of particle i (position pi): f(r, b, e, whole)
// with whole the row's candidate count and [b, e) the part of it walked.  With `prune`, a
// row whose cells lie farther than the kernel radius from pi in y and z is not walked, and
// the cell below or above in x is left out of a row when pi's sphere cannot reach it: a
// member j of that cell would satisfy x-distance >= (the distance from pi to its cell's face)
// and x-distance < sqrt(h^2 - dy^2 - dz^2), with dy, dz the y-z distances to the row's
// cells.  Distances are reduced (and the radius enlarged) by the margin P.prune_m, far above
// the rounding of positions and cell faces, so the walked candidates hold every member; they
// are the row's own candidates in the row's order, so the members and their order are the
// unpruned walk's.  A particle outside its own cell by more than the margin (clamped into
// the grid) walks whole rows.
template <class F>
__device__ __forceinline__ void tile_rows_pruned(const Params &P, const unsigned *__restrict__ start, float4 pi,
                                                 unsigned c, bool prune, F &&f) {
    const GridDev &g = P.g;
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
    const float m = P.prune_m, hm = P.h + m, hm2 = hm * hm;
    // offsets of pi in its cell: the distances to the faces of the cells below and above
    const float ux = pi.x - (g.minp[0] + (float)cx * g.len[0]);
    const float uy = pi.y - (g.minp[1] + (float)cy * g.len[1]);
    const float uz = pi.z - (g.minp[2] + (float)cz * g.len[2]);
    prune = prune && ux >= -m && ux <= g.len[0] + m && uy >= -m && uy <= g.len[1] + m && uz >= -m &&
            uz <= g.len[2] + m;
    const float ax_lo = ux - m, ax_hi = g.len[0] - ux - m;
    const float dy_lo = fmaxf(uy - m, 0.f), dy_hi = fmaxf(g.len[1] - uy - m, 0.f);
    const float dz_lo = fmaxf(uz - m, 0.f), dz_hi = fmaxf(g.len[2] - uz - m, 0.f);
    for (int z = z0; z <= z1; ++z) {
        const float dz = z < cz ? dz_lo : (z > cz ? dz_hi : 0.f);
        for (int y = y0; y <= y1; ++y) {
            const float dy = y < cy ? dy_lo : (y > cy ? dy_hi : 0.f);
            const unsigned row = (unsigned)y * (unsigned)nx + (unsigned)z * plane;
            const unsigned fb = __ldg(&start[row + (unsigned)x0]), fe = __ldg(&start[row + (unsigned)x1 + 1u]);
            unsigned b = fb, e = fe;
            if (prune) {
                const float r2 = hm2 - (dy * dy + dz * dz);
                if (r2 <= 0.f) {
                    e = fb;   // out of reach
                } else {
                    if (x0 < cx && ax_lo > 0.f && ax_lo * ax_lo >= r2) b = __ldg(&start[row + (unsigned)cx]);
                    if (x1 > cx && ax_hi > 0.f && ax_hi * ax_hi >= r2) e = __ldg(&start[row + (unsigned)cx + 1u]);
                    if (e < b) e = b;
                }
            }
            f((z - cz + 1) * 3 + (y - cy + 1), b, e, fe - fb);
        }
    }
}

// Number of candidates in the 27 cells of cell c.
__device__ __forceinline__ unsigned candidate_count(const GridDev &g, const unsigned *__restrict__ start,
                                                    unsigned c) {
    unsigned total = 0;
    tile_rows(g, start, c, [&](int, unsigned b, unsigned e) { total += e - b; });
    return total;
}

// Same visit order, for the density pass: f(j, base) with the list entry of slot j equal
// to j + base; *fits turns false when a range reaches past the 12-bit offset limit.
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
            if (kListRelative && e - lo > (unsigned)kOffLimit) *fits = false;
            for (unsigned j = b; j < e; ++j) f(j, base);
        }
    }
}



// For every member j != i of particle i's step-start neighbour set: use(fetch(j)).
// Members are processed NB at a time: the NB list entries and then the NB neighbour
// records are requested before any is used (entries past the end fetch particle i
// itself and are not used).  Wide particles re-test their candidates with the
// exact membership test at the step-start positions pos0.
template <int NB = kGatherBatch, bool SPLIT = false, class Fetch, class Use>
__device__ __forceinline__ void tile_members(const Params &P, const unsigned *__restrict__ start,
                                             const TileMap &T, const ListEntry *__restrict__ list,
                                             const int *__restrict__ nbr, const float4 *__restrict__ pos0,
                                             unsigned cellw, int i, Fetch &&fetch, Use &&use) {
    if (cellw & kWide) {
        if (candidate_count(P.g, start, cellw & ~kWide) > kMaxCandidates) return;
        const float4 pi = __ldg(&pos0[i]);
        tile_candidates(P.g, start, cellw & ~kWide, [&](unsigned j, int) {
            if (j == (unsigned)i) return;
            const float4 pj = __ldg(&pos0[j]);
            if (std_member(P, pi, pj, dist2(pi, pj))) use(fetch(j));
        });
        return;
    }
    const int cnt = __ldg(&nbr[i]) - 1;   // members other than i
    const size_t n = (size_t)P.n;
    const ListEntry *l = list + i;        // entry q + k of the group at l + k * n
    // SPLIT: whole groups without per-member predicates, then the partial group (a second
    // copy of `use`: measured faster for the small predicted-density body only)
    const int full = SPLIT ? cnt - cnt % NB : 0;
    int q = 0;
    for (; q < full; q += NB, l += NB * n) {
        unsigned j[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) j[k] = list_slot(T, __ldg(l + k * n));
        decltype(fetch(0u)) d[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) d[k] = fetch(j[k]);
#pragma unroll
        for (int k = 0; k < NB; k++) use(d[k]);
    }
    for (; q < cnt; q += NB, l += NB * n) {   // predicated groups (with SPLIT: the last one)
        unsigned j[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) j[k] = q + k < cnt ? list_slot(T, __ldg(l + k * n)) : (unsigned)i;
        decltype(fetch(0u)) d[NB];
#pragma unroll
        for (int k = 0; k < NB; k++) d[k] = fetch(j[k]);
#pragma unroll
        for (int k = 0; k < NB; k++)
            if (q + k < cnt) use(d[k]);
    }
}

}  // namespace bbg
