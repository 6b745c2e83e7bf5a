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
// It needs no context either: every byte it uses is a file-scope device
// array, reserved when the module loads.
//
// Scratch (g_scratch, kScratchBytes = 16 MiB + 256 B):
//   [0, 256)     accumulators: vertices, triangles, MC vertices.  They MUST
//                start at zero; every call clears them on its stream first.
//   [256, ...)   one uint4 per grid row (vertices, triangles, MC vertices, 0),
//                at most ISO_NOALLOC_MAX_ROWS = 2^20 rows (ny * nz); larger
//                grids are rejected with ISO_ERR_TOO_LARGE before any launch.
// Every row record is written before it is read, so only the accumulators
// need clearing.  Because the scratch is one array per device, calls on the
// same device must not overlap: two calls in flight at once (other streams
// or host threads) race on it.
//
// The first call on a device does the set-up, with that device current:
// cudaGetSymbolAddress of the scratch and a synchronous copy of the case
// tables into g_cases.  Later calls only enqueue a memset and three kernels.
#include <mutex>

#include "../../include/miniiso.h"
#include "case_table.h"
#include "iso_device.cuh"

namespace iso {
namespace {

constexpr long long kMaxRows = ISO_NOALLOC_MAX_ROWS;
constexpr size_t kAccumBytes = 256;
constexpr size_t kScratchBytes = kAccumBytes + 16 * (size_t)kMaxRows;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];
static __device__ CaseTables g_cases;

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
    __shared__ uint8_t s_ntris[256];
    __shared__ uint16_t s_cut[256];
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        s_ntris[c] = (uint8_t)iso_case_ntris(g_cases.tris[c]);
        s_cut[c] = g_cases.cut[c];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long r = (long long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
    if (r >= g.R) return;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const bool hasY = j < g.ny - 1, hasZ = k < g.nz - 1, cell = hasY && hasZ;
    const int jy = hasY ? j + 1 : j, kz = hasZ ? k + 1 : k;
    auto rowptr = [&](int kk, int jj) { return vol + ((long long)kk * g.ny + jj) * g.nx; };
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
        if (cell) {
            for (uint32_t act = active_cells(rw, evalid); act; act &= act - 1) {
                const int bit = __ffs(act) - 1;
                const int cs = cube_case(rw, bit);
                nt += s_ntris[cs];
                if (MC) nm += __popc(mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cut[cs]);
            }
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        nv += __shfl_xor_sync(0xffffffffu, nv, d);
        nt += __shfl_xor_sync(0xffffffffu, nt, d);
        if (MC) nm += __shfl_xor_sync(0xffffffffu, nm, d);
    }
    if (lane == 0) rows[r] = make_uint4(nv, nt, nm, 0u);
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

struct DeviceSetup {
    bool done = false;
    unsigned char* scratch = nullptr;
    int nsm = 0;
};
std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

void host_case_tables(CaseTables& t)
{
    for (int c = 0; c < 256; ++c) {
        const uint64_t w = kIsoCaseTris[c];
        t.tris[c] = w;
        uint16_t cut = 0;
        for (int e = 0; e < 12; ++e) {
            if (((c >> kIsoEdgeLo[e]) & 1) != ((c >> kIsoEdgeHi[e]) & 1)) cut |= (uint16_t)(1u << e);
        }
        t.cut[c] = cut;
        t.order[c] = 0;  // not used by the count
    }
}

// Once per device, with that device current.
iso_status setup_device(int dev, DeviceSetup*& out)
{
    if (dev < 0 || dev >= kMaxDevices) return ISO_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup& s = g_setup[dev];
    if (!s.done) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || p == nullptr) return ISO_ERR_CUDA;
        CaseTables h;
        host_case_tables(h);
        if (cudaMemcpyToSymbol(g_cases, &h, sizeof(CaseTables)) != cudaSuccess) return ISO_ERR_CUDA;
        int nsm = 0;
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ISO_ERR_CUDA;
        s.scratch = static_cast<unsigned char*>(p);
        s.nsm = nsm;
        s.done = true;
    }
    out = &s;
    return ISO_OK;
}

}  // namespace
}  // namespace iso

extern "C" iso_status iso_count_device_noalloc(iso_algorithm algo, const float* volume, const iso_grid* grid,
                                               float isoval, int64_t* counts, void* stream)
{
    using namespace iso;
    if (!volume || !grid || !counts) return ISO_ERR_INVALID_ARG;
    if (algo != ISO_FLYING_EDGES && algo != ISO_MARCHING_CUBES) return ISO_ERR_INVALID_ARG;
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
    if (g.R > kMaxRows) return ISO_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ISO_ERR_CUDA;
    DeviceSetup* su = nullptr;
    const iso_status st = setup_device(dev, su);
    if (st != ISO_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(su->scratch);
    uint4* rows = reinterpret_cast<uint4*>(su->scratch + kAccumBytes);
    if (cudaMemsetAsync(acc, 0, kAccumBytes, s) != cudaSuccess) return ISO_ERR_CUDA;
    const bool mc = algo == ISO_MARCHING_CUBES;
    if (g.nx >= 2 && g.ny >= 2 && g.nz >= 2) {  // a grid without cells has an empty mesh
        const unsigned blocks = (unsigned)((g.R + kThreads / 32 - 1) / (kThreads / 32));
        if (mc) k_na_rows<true><<<blocks, kThreads, 0, s>>>(volume, g, isoval, rows);
        else k_na_rows<false><<<blocks, kThreads, 0, s>>>(volume, g, isoval, rows);
        long long sum_blocks = (g.R + kThreads - 1) / kThreads;
        if (sum_blocks > 4ll * su->nsm) sum_blocks = 4ll * su->nsm;
        k_na_sum<<<(unsigned)sum_blocks, kThreads, 0, s>>>(rows, g.R, acc);
    }
    k_na_finish<<<1, 1, 0, s>>>(acc, mc ? 1 : 0, counts);
    return cudaGetLastError() == cudaSuccess ? ISO_OK : ISO_ERR_CUDA;
}
