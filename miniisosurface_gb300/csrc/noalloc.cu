// Allocation-free count entry point: iso_count_device_noalloc.
//
// The same output sizes as iso_count_device (passes 1-3 of
// flyingEdges/serial/FlyingEdgesAlgorithm.cpp:23-269, or the MC vertex and
// triangle counts of marchingCubes/serial/main.cpp:139-177), for callers
// that must not allocate device memory while they size a mesh:
//   * in-situ visualisation inside a solver that has reserved the device's
//     memory for its own pool, so a cudaMalloc would fail or evict it;
//   * an allocator asking for the size of a mesh before it carves the output
//     from its own arena, which cannot re-enter a general allocator;
//   * latency-bound loops sharing the device with other streams, where a
//     cudaFree (which synchronises the whole device) would stall them.
// It needs no context either: every byte it uses is one file-scope device
// array, which the device holds from the time this file's module loads until
// the process exits.  With CUDA's lazy module loading (the default) the module
// loads at the first call on a device, so a caller that is about to reserve
// the device's memory makes that first call before it does (a call on a
// one-point grid is enough), and before any stream capture.
//
// Scratch (g_scratch, kScratchBytes = 16 MiB + 256 B):
//   [0, 256)     accumulators: vertices, triangles, MC vertices.  They MUST
//                start at zero; every call clears them on its stream first.
//   [256, ...)   one uint4 per grid row (vertices, triangles, MC vertices, 0),
//                at most ISO_NOALLOC_MAX_ROWS = 2^20 rows (ny * nz); larger
//                grids are rejected with ISO_ERR_TOO_LARGE before any launch,
//                and so are rows of more than kMaxRowPoints points, whose
//                triangle count could pass 2^32.
// Every row record is written before it is read, so only the accumulators
// need clearing.  Because the scratch is one array per device, calls on the
// same device must not overlap: two calls in flight at once (other streams
// or host threads) race on it.
//
// No state is kept between calls: each call looks up the array's device
// address on the current device (cudaGetSymbolAddress, a host-side lookup
// once the module is loaded), so a call after a cudaDeviceReset uses the
// array of the freshly loaded module.  The counts need no case table: the
// triangles and Marching Cubes vertices of 32 cells at a time come from
// bit-parallel formulas over the cells' corner words (tris_of_word,
// mc_verts_of_word), the ones the count pass of the other entry points uses.
#include "../../include/miniiso.h"
#include "case_table.h"
#include "iso_device.cuh"

namespace iso {
namespace {

constexpr long long kMaxRows = ISO_NOALLOC_MAX_ROWS;
// A row's record holds 32-bit counts: at most 5 (nx - 1) triangles and
// 3 nx + 2 vertices, so rows are limited to (2^32 - 1) / 5 points.
constexpr long long kMaxRowPoints = ISO_NOALLOC_MAX_ROW_POINTS;
constexpr size_t kAccumBytes = 256;
constexpr size_t kScratchBytes = kAccumBytes + 16 * (size_t)kMaxRows;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Word c*32 + lane of a row, and word c*32 + 32 (uniform over the warp).
__device__ __forceinline__ void na_chunk(const float* __restrict__ row, bool ok, int c, int nx, int lane, float iso,
                                         uint32_t& word, uint32_t& next)
{
    word = 0u;
    next = 0u;
    for (int t = 0; t <= 32; ++t) {
        const long long i = 32ll * (32 * c + t) + lane;
        const bool in = ok && i < nx;
        const uint32_t m = __ballot_sync(0xffffffffu, in && __ldg(row + i) >= iso);
        if (t == lane) word = m;
        next = m;
    }
}

// One warp per grid row r = k*ny + j: the vertices it owns (cut x, y, z
// edges), the triangles of cell row (j,k) and, for MC, the vertices cell row
// (j,k) owns.  Writes rows[r].
template <bool MC>
__global__ void __launch_bounds__(kThreads) k_na_rows(const float* __restrict__ vol, Grid g, float iso,
                                                      uint4* __restrict__ rows)
{
    const int lane = threadIdx.x & 31;
    const long long r = (long long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    if (r >= g.R) return;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const bool hasY = j < g.ny - 1, hasZ = k < g.nz - 1, cell = hasY && hasZ;
    const int jy = hasY ? j + 1 : j, kz = hasZ ? k + 1 : k;
    auto rowptr = [&](int kk, int jj) { return vol + ((long long)kk * g.ny + jj) * g.nx; };
    // per lane at most 3 * 32 cut edges and 5 * 32 triangles per word, over at most 2^20 words
    uint32_t nv = 0, nt = 0, nm = 0;
    const int nchunks = (g.W + 31) / 32;
    for (int c = 0; c < nchunks; ++c) {
        RowWords rw;
        uint32_t na, nb, nc, nd;
        na_chunk(rowptr(k, j), true, c, g.nx, lane, iso, rw.a, na);
        na_chunk(rowptr(k, jy), hasY, c, g.nx, lane, iso, rw.b, nb);
        na_chunk(rowptr(kz, j), hasZ, c, g.nx, lane, iso, rw.c, nc);
        na_chunk(rowptr(kz, jy), cell, c, g.nx, lane, iso, rw.d, nd);
        const uint32_t da = __shfl_down_sync(0xffffffffu, rw.a, 1), db = __shfl_down_sync(0xffffffffu, rw.b, 1);
        const uint32_t dc = __shfl_down_sync(0xffffffffu, rw.c, 1), dd = __shfl_down_sync(0xffffffffu, rw.d, 1);
        rw.ash = (rw.a >> 1) | ((lane < 31 ? da : na) << 31);
        rw.bsh = (rw.b >> 1) | ((lane < 31 ? db : nb) << 31);
        rw.csh = (rw.c >> 1) | ((lane < 31 ? dc : nc) << 31);
        rw.dsh = (rw.d >> 1) | ((lane < 31 ? dd : nd) << 31);
        const int w = 32 * c + lane;
        const uint32_t evalid = validmask(w, g.nx - 1);
        const uint32_t pvalid = validmask(w, g.nx);
        nv += __popc((rw.a ^ rw.ash) & evalid);
        if (hasY) nv += __popc((rw.a ^ rw.b) & pvalid);
        if (hasZ) nv += __popc((rw.a ^ rw.c) & pvalid);
        if (cell) {  // the word's 32 cells at once; corners 0..7 = a ash bsh b c csh dsh d
            nt += tris_of_word(rw.a, rw.ash, rw.bsh, rw.b, rw.c, rw.csh, rw.dsh, rw.d, evalid);
            if (MC)
                nm += mc_verts_of_word(rw.a, rw.ash, rw.bsh, rw.b, rw.c, rw.csh, rw.dsh, rw.d, evalid, j == 0, k == 0,
                                       w == 0);
        }
    }
    // row totals in 64 bits (32 lanes), stored as 32-bit counts: rows are limited to kMaxRowPoints points
    unsigned long long v = nv, t = nt, m = nm;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, d);
        t += __shfl_xor_sync(0xffffffffu, t, d);
        if (MC) m += __shfl_xor_sync(0xffffffffu, m, d);
    }
    if (lane == 0) rows[r] = make_uint4((uint32_t)v, (uint32_t)t, (uint32_t)m, 0u);
}

// Sums of the row records into the accumulators (which start at zero).
__global__ void __launch_bounds__(kThreads) k_na_sum(const uint4* __restrict__ rows, long long R,
                                                     unsigned long long* __restrict__ acc)
{
    __shared__ unsigned long long s[3][kThreads / 32];
    unsigned long long v = 0, t = 0, m = 0;
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (long long)gridDim.x * blockDim.x) {
        const uint4 c = rows[r];
        v += c.x;
        t += c.y;
        m += c.z;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, d);
        t += __shfl_xor_sync(0xffffffffu, t, d);
        m += __shfl_xor_sync(0xffffffffu, m, d);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][warp] = v;
        s[1][warp] = t;
        s[2][warp] = m;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long x = 0;
        for (int q = 0; q < kThreads / 32; ++q) x += s[threadIdx.x][q];
        atomicAdd(&acc[threadIdx.x], x);
    }
}

__global__ void k_na_finish(const unsigned long long* __restrict__ acc, int mc, int64_t* __restrict__ out)
{
    out[0] = (int64_t)acc[mc ? 2 : 0];
    out[1] = (int64_t)acc[1];
}

// The scratch array's address on the current device.  Looked up on every
// call: the lookup is cheap once the module is loaded, and nothing cached can
// outlive a cudaDeviceReset.
cudaError_t scratch_address(unsigned char*& out)
{
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    out = static_cast<unsigned char*>(p);
    return e != cudaSuccess ? e : (p ? cudaSuccess : cudaErrorInvalidSymbol);
}

// A kThreads-wide launch that returns its own status.
template <typename... Params, typename... Args>
cudaError_t launch(void (*kern)(Params...), unsigned blocks, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace
}  // namespace iso

extern "C" iso_status iso_count_device_noalloc(iso_algorithm algo, const float* volume, const iso_grid* grid,
                                               float isoval, int64_t* counts, void* stream)
{
    using namespace iso;
    if (!volume || !grid || !counts) return ISO_ERR_INVALID_ARG;
    // ISO_MC_DUPFREE numbers the same vertices as ISO_MARCHING_CUBES in another order: the same counts
    if (algo != ISO_FLYING_EDGES && algo != ISO_MARCHING_CUBES && algo != ISO_MC_DUPFREE) return ISO_ERR_INVALID_ARG;
    Grid g{};
    for (int a = 0; a < 3; ++a) {
        if (grid->dims[a] < 1 || grid->dims[a] > (1ll << 30)) return ISO_ERR_INVALID_ARG;
    }
    g.nx = (int)grid->dims[0];
    g.ny = (int)grid->dims[1];
    g.nz = (int)grid->dims[2];
    g.W = (g.nx + 31) / 32;
    g.R = (long long)g.ny * g.nz;
    for (int a = 0; a < 3; ++a) {
        g.sp[a] = grid->spacing[a];
        g.zp[a] = grid->origin[a];
    }
    if (g.R > kMaxRows || g.nx > kMaxRowPoints) return ISO_ERR_TOO_LARGE;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ISO_ERR_CUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ISO_ERR_CUDA;
    unsigned char* scratch = nullptr;
    if (scratch_address(scratch) != cudaSuccess) return ISO_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(scratch);
    uint4* rows = reinterpret_cast<uint4*>(scratch + kAccumBytes);
    // each launch's own status, so an earlier, unrelated error on this thread is neither reported nor cleared
    if (cudaMemsetAsync(acc, 0, kAccumBytes, s) != cudaSuccess) return ISO_ERR_CUDA;
    const bool mc = algo != ISO_FLYING_EDGES;
    if (g.nx >= 2 && g.ny >= 2 && g.nz >= 2) {  // a grid without cells has an empty mesh
        const unsigned blocks = (unsigned)((g.R + kThreads / 32 - 1) / (kThreads / 32));
        const cudaError_t e = mc ? launch(k_na_rows<true>, blocks, s, volume, g, isoval, rows)
                                 : launch(k_na_rows<false>, blocks, s, volume, g, isoval, rows);
        if (e != cudaSuccess) return ISO_ERR_CUDA;
        long long sum_blocks = (g.R + kThreads - 1) / kThreads;
        if (sum_blocks > 4ll * nsm) sum_blocks = 4ll * nsm;
        if (launch(k_na_sum, (unsigned)sum_blocks, s, (const uint4*)rows, g.R, acc) != cudaSuccess) return ISO_ERR_CUDA;
    }
    cudaLaunchConfig_t one = {};
    one.gridDim = dim3(1);
    one.blockDim = dim3(1);
    one.stream = s;
    if (cudaLaunchKernelEx(&one, k_na_finish, (const unsigned long long*)acc, mc ? 1 : 0, counts) != cudaSuccess)
        return ISO_ERR_CUDA;
    return ISO_OK;
}
