// noalloc.cu -- grid sort for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc: a host application that owns
// the device-memory budget (a fixed pool carved out at start-up, or an allocator that
// other code must not bypass) and loads this library as a plugin, or code that runs
// where allocation is forbidden.  bbg_grid_sort_noalloc serves them: it computes the
// same grid as a solver's bbg_update_grid_distribution + bbg_dump_grid (exact reference
// hash, stable counting sort by (cell id, particle index)) on buffers the caller owns,
// and keeps its own scratch in one file-scope __device__ array of fixed size instead of
// allocating.
//
// Rules of use:
//  - A call outside stream capture looks up the scratch array's device address on the
//    current device (cudaGetSymbolAddress) every time, so a device reset between calls
//    (which unloads the module and frees the array) is picked up; a call inside a
//    capture uses the address an earlier uncaptured call on that device found, so make
//    the first call on a device outside any stream capture.
//  - Every call on a device shares the one scratch array, and it keeps the previous
//    call's contents (this file clears what must start at zero).  Calls whose GPU work
//    overlaps -- on different streams, or from different host threads -- race on it;
//    serialise them.
//  - The array occupies BBG_NOALLOC_SCRATCH_BYTES on every GPU that loads the library,
//    until the process exits.
#include "../../include/bbg.h"
#include "bbg_kernels.h"
#include "host_math.h"

#include <mutex>

namespace bbg {
namespace {

constexpr unsigned kMaxP = BBG_NOALLOC_MAX_PARTICLES;
constexpr unsigned kMaxC = BBG_NOALLOC_MAX_CELLS;
constexpr unsigned kPartialWords = ((kMaxC + 2047u) / 2048u + 2u + 1u) & ~1u;   // even
// word layout: counts[kMaxC] | partials | arrival index[kMaxP] | cell[kMaxP] | pairs[2 kMaxP]
constexpr size_t kWords = (size_t)kMaxC + kPartialWords + 2u * (size_t)kMaxP + 2u * (size_t)kMaxP;
static_assert(kWords * 4 == BBG_NOALLOC_SCRATCH_BYTES, "scratch size must match the header");

static __device__ __align__(256) unsigned g_scratch[kWords];

constexpr int kThreads = 256;
static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

__global__ void __launch_bounds__(kThreads)
k_na_hash_count(GridDev g, float iz, const float *__restrict__ xyz, int n,
                unsigned *__restrict__ cell_old, unsigned *__restrict__ sub,
                unsigned *__restrict__ count, unsigned *__restrict__ out_of_grid) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    unsigned bad = 0, c = 0xffffffffu;
    if (valid) c = grid_hash(g, make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.f), iz, &bad);
    // particles outside the grid are clamped into its edge cells (as the solver's grid);
    // the caller's counter, when given, receives how many
    const unsigned outside = __ballot_sync(0xffffffffu, valid && bad);
    if (out_of_grid && (threadIdx.x & 31) == 0 && outside) atomicAdd(out_of_grid, (unsigned)__popc(outside));
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    const unsigned peers = __match_any_sync(mask, c);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    const unsigned rank = __popc(peers & ((1u << lane) - 1u));
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&count[c], (unsigned)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    sub[i] = base + rank;
    cell_old[i] = c;
}

__global__ void __launch_bounds__(kThreads)
k_na_place(int n, const unsigned *__restrict__ cell_old, const unsigned *__restrict__ sub,
           const unsigned *__restrict__ start, uint2 *__restrict__ pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pairs[start[cell_old[i]] + sub[i]] = make_uint2((unsigned)i, cell_old[i]);
}

__global__ void __launch_bounds__(kThreads)
k_na_rank(int n, const uint2 *__restrict__ pairs, const unsigned *__restrict__ start,
          unsigned *__restrict__ cell_of, unsigned *__restrict__ sorted_ids) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint2 e = pairs[t];   // (particle index, cell)
    const unsigned a = start[e.y], b = start[e.y + 1];
    unsigned dst = (unsigned)t;   // arrival order in a cell past the rank cap, as the solver
    if (b - a <= kRankCap) {
        unsigned rank = 0;
        for (unsigned q = a; q < b; ++q) rank += (pairs[q].x < e.x) ? 1u : 0u;
        dst = a + rank;
    }
    sorted_ids[dst] = e.x;
    cell_of[e.x] = e.y;
}

std::mutex g_mutex;
unsigned *g_ptr[256] = {nullptr};

// Device address of g_scratch on the current device.  Outside stream capture it is looked
// up on every call (a device reset frees the module's array and a later load may place it
// elsewhere); inside a capture, where the lookup may not be legal, the address the last
// uncaptured call on this device found is used.
int scratch_for_current_device(cudaStream_t stream, unsigned **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 256)
        return set_error(BBG_ERR_NO_DEVICE, "bbg_grid_sort_noalloc: no current CUDA device (%s)",
                         cudaGetErrorString(e));
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess)
        return set_error(BBG_ERR_CUDA, "bbg_grid_sort_noalloc: cudaStreamIsCapturing: %s", cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(g_mutex);
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p)
            return set_error(BBG_ERR_CUDA, "bbg_grid_sort_noalloc: cudaGetSymbolAddress: %s",
                             cudaGetErrorString(e));
        g_ptr[dev] = (unsigned *)p;
    } else if (!g_ptr[dev]) {
        return set_error(BBG_ERR_STATE,
                         "bbg_grid_sort_noalloc: the first call on a device must be outside stream capture");
    }
    *out = g_ptr[dev];
    return BBG_OK;
}

}  // namespace
}  // namespace bbg

extern "C" bbg_status bbg_grid_sort_noalloc(const float *d_pos, int n, const double domain_min[3],
                                            const double domain_max[3], double spacing,
                                            double spacing_scale, uint32_t *d_cell_of,
                                            uint32_t *d_sorted_ids, uint32_t *d_cell_start,
                                            uint32_t *d_out_of_grid, void *stream) {
    using namespace bbg;
    if (!d_pos || !d_cell_of || !d_sorted_ids || !d_cell_start || !domain_min || !domain_max)
        return set_error(BBG_ERR_INVALID_ARGUMENT, "bbg_grid_sort_noalloc: null pointer argument");
    if (n <= 0 || !(spacing > 0) || !(spacing_scale > 0))
        return set_error(BBG_ERR_INVALID_ARGUMENT, "bbg_grid_sort_noalloc: need n > 0, spacing > 0, scale > 0");
    if ((unsigned)n > kMaxP)
        return set_error(BBG_ERR_CAPACITY,
                         "bbg_grid_sort_noalloc: %d particles exceed the fixed scratch limit of %u",
                         n, kMaxP);
    for (int k = 0; k < 3; k++)
        if (!(domain_max[k] > domain_min[k]))
            return set_error(BBG_ERR_INVALID_ARGUMENT, "bbg_grid_sort_noalloc: empty domain on axis %d", k);
    GridDev g;
    int dims[3];
    build_grid(domain_min, domain_max, spacing, spacing_scale, dims, g.minp, g.len, g.bmin, g.bmax);
    const unsigned long long cells = (unsigned long long)dims[0] * dims[1] * dims[2];
    if (cells == 0 || cells > kMaxC)
        return set_error(BBG_ERR_CAPACITY,
                         "bbg_grid_sort_noalloc: grid of %llu cells exceeds the fixed scratch limit of %u",
                         cells, kMaxC);
    g.nx = dims[0];
    g.ny = dims[1];
    g.nz = dims[2];
    g.total = (unsigned)cells;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned *base = nullptr;
    if (int r = scratch_for_current_device(s, &base)) return r;
    unsigned *count = base;
    unsigned *partials = count + kMaxC;
    unsigned *sub = partials + kPartialWords;
    unsigned *cell_old = sub + kMaxP;
    uint2 *pairs = reinterpret_cast<uint2 *>(cell_old + kMaxP);
    // the histogram (and the caller's counter) must start at zero; everything else is
    // fully overwritten
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned) * (size_t)cells, s);
    if (e == cudaSuccess && d_out_of_grid) e = cudaMemsetAsync(d_out_of_grid, 0, sizeof(unsigned), s);
    if (e != cudaSuccess)
        return set_error(BBG_ERR_CUDA, "bbg_grid_sort_noalloc: %s", cudaGetErrorString(e));
    const float iz = float_above(1e-8);
    k_na_hash_count<<<blocks_for(n, kThreads), kThreads, 0, s>>>(g, iz, d_pos, n, cell_old, sub, count,
                                                                  d_out_of_grid);
    launch_cell_scan(count, (unsigned)cells, partials, d_cell_start, s);
    k_na_place<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, cell_old, sub, d_cell_start, pairs);
    k_na_rank<<<blocks_for(n, kThreads), kThreads, 0, s>>>(n, pairs, d_cell_start, d_cell_of,
                                                           d_sorted_ids);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(BBG_ERR_CUDA, "bbg_grid_sort_noalloc: %s", cudaGetErrorString(e));
    return BBG_OK;
}
