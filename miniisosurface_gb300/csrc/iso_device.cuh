// Device-side helpers shared by the Flying Edges and Marching Cubes kernels.
//
// Data layout in HBM (one extraction):
//   volume  float32[nz][ny][nx]                  x fastest (Image3D.h:26-85)
//   rowcnt  uint4[R]       per grid row r = k*ny + j (R = ny*nz): cut x / y / z
//                          edges owned by the row, triangles of cell row (j,k)
//   trims   uint2[R]       xl, xr of the row (FlyingEdgesAlgorithm.cpp:47-65)
//   mccnt   uint32[R]      marching cubes: vertices owned by cell row (j,k)
//   starts  u64[3][R]      first vertex / triangle / mc vertex of each row
//                          (exclusive scans of the counts in row order)
//   bits    uint32[R][W]   W = ceil(nx/32); bit i of row r = value >= isovalue
//                          (written only when a row-wise kernel needs it)
//   totals  u64[4]         vertices, triangles, mc vertices, device status
//
// All interpolation arithmetic goes through the _rn intrinsics so that no
// multiply-add is ever contracted: that reproduces the float32 results of the
// reference CPU code bit for bit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "case_table.h"

namespace iso {

constexpr int kTileRows = 256;     // grid rows per count/scan tile
constexpr int kThreads = 256;      // threads per CTA of the row kernels

struct Grid {
    int nx, ny, nz;
    int W;                 // 32-bit words per bit row
    long long R;           // grid rows of the window = ny * (ke - kr)
    float sp[3], zp[3];
    // z window (a slab of a decomposition; the whole grid by default): the
    // volume pointer holds planes from kd on, the per-row scratch covers
    // planes [kr, ke), row (j, k) at index (k - kr) * ny + j.
    int kd, kr, ke;
};

// Per-case data derived from the packed triangle table when a context is
// created, resident in device memory and staged into shared memory per CTA.
struct CaseTables {
    uint64_t tris[256];    // packed triangle lists (case_table.h)
    uint64_t order[256];   // cube edges in order of first appearance in the
                           // triangle list, packed like tris (count in 60..63)
    uint16_t cut[256];     // 12-bit mask of the cut cube edges of the case
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ uint32_t lowmask(int pos)  // bits [0, pos), pos in [0, 32]
{
    return (uint32_t)((1ull << pos) - 1ull);
}

// Mask of valid bit positions of word w when only indices < limit exist.
__device__ __forceinline__ uint32_t validmask(int w, int limit)
{
    int rem = limit - 32 * w;
    if (rem >= 32) return 0xffffffffu;
    if (rem <= 0) return 0u;
    return lowmask(rem);
}

// Group-level (width G lanes) inclusive scan.
template <int G>
__device__ __forceinline__ uint32_t group_incl_scan(uint32_t v, int lig, unsigned mask)
{
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
        uint32_t t = __shfl_up_sync(mask, v, d, G);
        if (lig >= d) v += t;
    }
    return v;
}

template <int G>
__device__ __forceinline__ uint32_t group_bcast(uint32_t v, int src, unsigned mask)
{
    return __shfl_sync(mask, v, src, G);
}

template <int G>
__device__ __forceinline__ uint32_t group_min(uint32_t v, unsigned mask)
{
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = min(v, __shfl_xor_sync(mask, v, d, G));
    return v;
}

template <int G>
__device__ __forceinline__ uint32_t group_max(uint32_t v, unsigned mask)
{
#pragma unroll
    for (int d = G / 2; d > 0; d >>= 1) v = max(v, __shfl_xor_sync(mask, v, d, G));
    return v;
}

// Value of the volume at grid point (i, j, k).
__device__ __forceinline__ float vload(const float* __restrict__ vol, const Grid& g, int i, int j, int k)
{
    return __ldg(vol + ((long long)k * g.ny + j) * g.nx + i);
}

// One component of the (negated, unnormalised) gradient at a grid point along
// one axis: Image3D::computeGradient (flyingEdges/util/Image3D.cpp:116-188).
// prev/here/next are the values at p-1, p, p+1 along that axis.
__device__ __forceinline__ float grad_component(float prev, float here, float next, int p, int n, float sp)
{
    if (p == 0) return fdiv(fsub(here, next), sp);
    if (p == n - 1) return fdiv(fsub(prev, here), sp);
    return fdiv(fsub(prev, next), fmul(2.0f, sp));
}

__device__ __forceinline__ float3 gradient_at(const float* __restrict__ vol, const Grid& g, int i, int j, int k)
{
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    const float* p = vol + (long long)k * sz + (long long)j * sy + i;
    float here = __ldg(p);
    float xm = i > 0 ? __ldg(p - 1) : 0.f, xp = i < g.nx - 1 ? __ldg(p + 1) : 0.f;
    float ym = j > 0 ? __ldg(p - sy) : 0.f, yp = j < g.ny - 1 ? __ldg(p + sy) : 0.f;
    float zm = k > 0 ? __ldg(p - sz) : 0.f, zp = k < g.nz - 1 ? __ldg(p + sz) : 0.f;
    float3 r;
    r.x = grad_component(xm, here, xp, i, g.nx, g.sp[0]);
    r.y = grad_component(ym, here, yp, j, g.ny, g.sp[1]);
    r.z = grad_component(zm, here, zp, k, g.nz, g.sp[2]);
    return r;
}

// Coordinate of grid index p along axis a when the cube that computes the
// vertex has base index `base` and the point is at offset p-base (0 or 1) from
// it: Image3D::getPosCube (flyingEdges/util/Image3D.cpp:45-87) forms
// zeroPos + base*spacing and adds spacing once for the far corner.
__device__ __forceinline__ float cube_coord(int base, int off, float zp, float sp)
{
    float c = fadd(zp, fmul((float)base, sp));
    return off ? fadd(c, sp) : c;
}

// interpolate() of FlyingEdgesAlgorithm.cpp:637-647 for one component.
__device__ __forceinline__ float lerp_ref(float a, float b, float w)
{
    return fadd(a, fmul(w, fsub(b, a)));
}

// Point and normal of the vertex on the edge from grid point (i,j,k) along
// `axis` (0=x,1=y,2=z), computed by the cube whose base is (ci,cj,ck).
// The edge runs from its lower to its higher grid point, as every entry of
// edgeVertices does (MarchingCubesTables.h:563).
__device__ __forceinline__ void edge_vertex(const float* __restrict__ vol, const Grid& g, float iso,
                                            int axis, int i, int j, int k, int ci, int cj, int ck,
                                            float3& pos, float3& nrm)
{
    const int i1 = i + (axis == 0), j1 = j + (axis == 1), k1 = k + (axis == 2);
    const float v0 = vload(vol, g, i, j, k);
    const float v1 = vload(vol, g, i1, j1, k1);
    const float w = fdiv(fsub(iso, v0), fsub(v1, v0));
    const float ax0 = cube_coord(ci, i - ci, g.zp[0], g.sp[0]);
    const float ay0 = cube_coord(cj, j - cj, g.zp[1], g.sp[1]);
    const float az0 = cube_coord(ck, k - ck, g.zp[2], g.sp[2]);
    const float ax1 = cube_coord(ci, i1 - ci, g.zp[0], g.sp[0]);
    const float ay1 = cube_coord(cj, j1 - cj, g.zp[1], g.sp[1]);
    const float az1 = cube_coord(ck, k1 - ck, g.zp[2], g.sp[2]);
    pos.x = lerp_ref(ax0, ax1, w);
    pos.y = lerp_ref(ay0, ay1, w);
    pos.z = lerp_ref(az0, az1, w);
    const float3 g0 = gradient_at(vol, g, i, j, k);
    const float3 g1 = gradient_at(vol, g, i1, j1, k1);
    nrm.x = lerp_ref(g0.x, g1.x, w);
    nrm.y = lerp_ref(g0.y, g1.y, w);
    nrm.z = lerp_ref(g0.z, g1.z, w);
}

// ---------------------------------------------------------------------------
// Row context: the four bit rows a cell row touches, one 32-bit word per lane.
//   A = (j,k)  B = (j+1,k)  C = (j,k+1)  D = (j+1,k+1)
// "sh" words hold bit i+1 at position i (the next word supplies bit 31).
// ---------------------------------------------------------------------------
struct RowWords {
    uint32_t a, b, c, d;
    uint32_t ash, bsh, csh, dsh;
};

__device__ __forceinline__ uint32_t load_word(const uint32_t* __restrict__ row, int w, int W, bool ok)
{
    return (ok && w < W) ? __ldg(row + w) : 0u;
}

__device__ __forceinline__ RowWords load_row_words(const uint32_t* __restrict__ bits, const Grid& g,
                                                   long long r, int w, bool valid, bool hasY, bool hasZ)
{
    RowWords rw;
    const uint32_t* A = bits + r * g.W;
    const uint32_t* B = A + g.W;
    const uint32_t* C = A + (long long)g.ny * g.W;
    const uint32_t* D = C + g.W;
    const bool cell = hasY && hasZ;
    rw.a = load_word(A, w, g.W, valid);
    rw.b = load_word(B, w, g.W, hasY);
    rw.c = load_word(C, w, g.W, hasZ);
    rw.d = load_word(D, w, g.W, cell);
    const uint32_t an = load_word(A, w + 1, g.W, valid);
    const uint32_t bn = load_word(B, w + 1, g.W, hasY);
    const uint32_t cn = load_word(C, w + 1, g.W, hasZ);
    const uint32_t dn = load_word(D, w + 1, g.W, cell);
    rw.ash = (rw.a >> 1) | (an << 31);
    rw.bsh = (rw.b >> 1) | (bn << 31);
    rw.csh = (rw.c >> 1) | (cn << 31);
    rw.dsh = (rw.d >> 1) | (dn << 31);
    return rw;
}

// Cells i of the word whose 8 corners are not all on the same side.
__device__ __forceinline__ uint32_t active_cells(const RowWords& rw, uint32_t cellvalid)
{
    const uint32_t and4 = rw.a & rw.b & rw.c & rw.d;
    const uint32_t and4s = rw.ash & rw.bsh & rw.csh & rw.dsh;
    const uint32_t or4 = rw.a | rw.b | rw.c | rw.d;
    const uint32_t or4s = rw.ash | rw.bsh | rw.csh | rw.dsh;
    return ~((and4 & and4s) | ~(or4 | or4s)) & cellvalid;
}

// Cube case of cell i of the word: bit v set <=> corner v >= isovalue
// (calcCubeCase, FlyingEdgesAlgorithm.cpp:576-604; findCaseId, util.h:24-42).
__device__ __forceinline__ int cube_case(const RowWords& rw, int bit)
{
    return (int)(((rw.a >> bit) & 1u) | (((rw.ash >> bit) & 1u) << 1) | (((rw.bsh >> bit) & 1u) << 2) |
                 (((rw.b >> bit) & 1u) << 3) | (((rw.c >> bit) & 1u) << 4) | (((rw.csh >> bit) & 1u) << 5) |
                 (((rw.dsh >> bit) & 1u) << 6) | (((rw.d >> bit) & 1u) << 7));
}

// The eight cut masks of a cell row (one word of each), from which the
// Flying Edges vertex id of any of the 12 edges of a cell is a popc rank.
struct CutMasks {
    uint32_t xA, xB, xC, xD;   // x-edges of rows A..D, bit i = edge (i, i+1)
    uint32_t yA, yC;           // y-edges A->B and C->D, bit i = point i
    uint32_t zA, zB;           // z-edges A->C and B->D, bit i = point i
};

__device__ __forceinline__ CutMasks cut_masks(const RowWords& rw, uint32_t evalid, uint32_t pvalid, bool hasY,
                                              bool hasZ)
{
    const bool cell = hasY && hasZ;
    CutMasks m;
    m.xA = (rw.a ^ rw.ash) & evalid;
    m.yA = hasY ? ((rw.a ^ rw.b) & pvalid) : 0u;
    m.zA = hasZ ? ((rw.a ^ rw.c) & pvalid) : 0u;
    m.xB = cell ? ((rw.b ^ rw.bsh) & evalid) : 0u;
    m.xC = cell ? ((rw.c ^ rw.csh) & evalid) : 0u;
    m.xD = cell ? ((rw.d ^ rw.dsh) & evalid) : 0u;
    m.yC = cell ? ((rw.c ^ rw.d) & pvalid) : 0u;
    m.zB = cell ? ((rw.b ^ rw.d) & pvalid) : 0u;
    return m;
}

// Flying Edges vertex ids of the first cut edge of each mask at this word
// (row start + prefix inside the row).
struct CutBases {
    unsigned long long xA, xB, xC, xD, yA, yC, zA, zB;
};

// Flying Edges vertex id of cube edge e of cell `bit` of the word, without
// branches (lanes of a warp usually ask for different edges):
//   e : 0  1  2  3  4  5  6  7  8  9  10 11
//   mask xA yA xB yA xC yC xD yC zA zA zB zB    (index 0..7 below)
//   +1  .  1  .  .  .  1  .  .  .  1  .  1      (edge at point i+1)
__device__ __forceinline__ unsigned long long fe_edge_id(const CutMasks& m, const CutBases& b, int e, int bit)
{
    // mask index per edge: xA=0 xB=1 xC=2 xD=3 yA=4 yC=5 zA=6 zB=7
    const int sel = (int)((0x776653524140ull >> (4 * e)) & 7u);
    const int off = (0xA22 >> e) & 1;
    const uint32_t mk = sel == 0 ? m.xA : sel == 1 ? m.xB : sel == 2 ? m.xC : sel == 3 ? m.xD
                      : sel == 4 ? m.yA : sel == 5 ? m.yC : sel == 6 ? m.zA : m.zB;
    const unsigned long long bs = sel == 0 ? b.xA : sel == 1 ? b.xB : sel == 2 ? b.xC : sel == 3 ? b.xD
                                : sel == 4 ? b.yA : sel == 5 ? b.yC : sel == 6 ? b.zA : b.zB;
    return bs + __popc(mk & lowmask(bit + off));
}

// Walks the flattened index f = tid, tid + step, tid + 2*step, ... of a
// (row, column) grid with `ncol` columns without dividing in the loop.
struct RowColWalk {
    int row, col, drow, dcol, ncol;
    __device__ __forceinline__ RowColWalk(int start, int step, int ncol_)
        : row(start / ncol_), col(start % ncol_), drow(step / ncol_), dcol(step % ncol_), ncol(ncol_) {}
    __device__ __forceinline__ void advance()
    {
        row += drow;
        col += dcol;
        if (col >= ncol) {
            col -= ncol;
            ++row;
        }
    }
};

// Bit mask "value >= iso" of rows [0, nrows) of nx values each (row stride
// nx) into dst[row * W + w].  All threads of the CTA take part; SHARED
// selects a shared-memory source (plain loads) or a global one (__ldg).
template <bool VEC4, bool SHARED>
__device__ __forceinline__ void classify_block(const float* __restrict__ src, int nx, int W, int nrows, float iso,
                                               uint32_t* __restrict__ dst)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (VEC4) {
        const int nq = nx >> 2, nq8 = (nq + 7) & ~7;
        constexpr int U = 4;
        RowColWalk it(tid, kThreads, nq8);
        const int total = nrows * nq8;
        for (int f0 = 0; f0 < total; f0 += U * kThreads) {
            float4 v[U];
            RowColWalk at = it;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = at.row < nrows && at.col < nq;
                const float4* p = reinterpret_cast<const float4*>(src + (size_t)at.row * nx) + at.col;
                v[u] = ok ? (SHARED ? *p : __ldg(p)) : make_float4(0.f, 0.f, 0.f, 0.f);
                at.advance();
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = it.row < nrows && it.col < nq;
                const uint32_t nib = ok ? ((uint32_t)(v[u].x >= iso) | ((uint32_t)(v[u].y >= iso) << 1) |
                                           ((uint32_t)(v[u].z >= iso) << 2) | ((uint32_t)(v[u].w >= iso) << 3))
                                        : 0u;
                uint32_t word = nib << (4 * (lane & 7));
                word |= __shfl_xor_sync(0xffffffffu, word, 1);
                word |= __shfl_xor_sync(0xffffffffu, word, 2);
                word |= __shfl_xor_sync(0xffffffffu, word, 4);
                if ((lane & 7) == 0 && ok) dst[it.row * W + (it.col >> 3)] = word;
                it.advance();
            }
        }
    } else {
        constexpr int U = 4, NW = kThreads / 32;
        RowColWalk it(warp, NW, W);
        const int total = nrows * W;
        for (int f0 = 0; f0 < total; f0 += U * NW) {
            float v[U];
            RowColWalk at = it;
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = 32 * at.col + lane;
                const bool ok = at.row < nrows && i < nx;
                const float* p = src + (size_t)at.row * nx + i;
                v[u] = ok ? (SHARED ? *p : __ldg(p)) : 0.f;
                at.advance();
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int i = 32 * it.col + lane;
                const bool ok = it.row < nrows && i < nx;
                const uint32_t word = __ballot_sync(0xffffffffu, ok && v[u] >= iso);
                if (lane == 0 && it.row < nrows) dst[it.row * W + it.col] = word;
                it.advance();
            }
        }
    }
}

// q = x / d for 0 <= x < 2^22 using a float reciprocal inv = 1/d and one
// correction step (no integer division in hot loops).
__device__ __forceinline__ int fastdiv(int x, int d, float inv)
{
    int q = __float2int_rz((float)x * inv);
    if (q * d > x) --q;
    else if ((q + 1) * d <= x) ++q;
    return q;
}

// Low grid point and axis of cube edge e of cell (0,0,0).
__device__ __forceinline__ void cube_edge_geometry(int e, int& dx, int& dy, int& dz, int& axis)
{
    // e:      0  1  2  3  4  5  6  7  8  9 10 11
    // dx:     0  1  0  0  0  1  0  0  0  1  0  1
    // dy:     0  0  1  0  0  0  1  0  0  0  1  1
    // dz:     0  0  0  0  1  1  1  1  0  0  0  0
    // axis:   x  y  x  y  x  y  x  y  z  z  z  z
    dx = (0xA22 >> e) & 1;
    dy = (0xC44 >> e) & 1;
    dz = (0x0F0 >> e) & 1;
    axis = e >= 8 ? 2 : (e & 1);
}

// Shared memory copy of the case tables.
struct SharedCases {
    uint64_t tris[256];
    uint64_t order[256];
    uint16_t cut[256];
};

__device__ __forceinline__ void stage_cases(SharedCases& s, const CaseTables* __restrict__ t, bool need_order)
{
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        s.tris[c] = t->tris[c];
        if (need_order) {
            s.order[c] = t->order[c];
            s.cut[c] = t->cut[c];
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Asynchronous global -> shared copies (TMA bulk engine or cp.async) with
// mbarrier completion, and bounded waits.
// ---------------------------------------------------------------------------
constexpr unsigned kWaitLimit = 1u << 22;   // try_wait rounds before giving up
constexpr unsigned long long kStatusTimeout = 6;  // ISO_ERR_TIMEOUT

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// One bulk copy (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

#ifdef ISO_WAIT_STATS
// Diagnostic build only: try_wait rounds and cycles spent in mbar_wait (per
// translation unit), read back through the accessor each unit defines.
__device__ unsigned long long g_wait_rounds, g_wait_cycles, g_wait_calls;
#define ISO_WAIT_STATS_ACCESSOR(name)                                                  \
    extern "C" void name(unsigned long long* o)                                      \
    {                                                                                  \
        cudaMemcpyFromSymbol(o, iso::g_wait_rounds, 8);                                \
        cudaMemcpyFromSymbol(o + 1, iso::g_wait_cycles, 8);                            \
        cudaMemcpyFromSymbol(o + 2, iso::g_wait_calls, 8);                             \
        unsigned long long z = 0;                                                      \
        cudaMemcpyToSymbol(iso::g_wait_rounds, &z, 8);                                 \
        cudaMemcpyToSymbol(iso::g_wait_cycles, &z, 8);                                 \
        cudaMemcpyToSymbol(iso::g_wait_calls, &z, 8);                                  \
    }
#else
#define ISO_WAIT_STATS_ACCESSOR(name)
#endif

// Bounded wait for phase `parity` of `bar`.  Returns false after kWaitLimit
// rounds (the caller records a timeout status and stops issuing work).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity)
{
#ifdef ISO_WAIT_STATS
    const long long t0 = clock64();
    for (unsigned n = 0; n < kWaitLimit; ++n) {
        if (mbar_try_wait(bar, parity)) {
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&g_wait_rounds, (unsigned long long)n + 1);
                atomicAdd(&g_wait_cycles, (unsigned long long)(clock64() - t0));
                atomicAdd(&g_wait_calls, 1ull);
            }
            return true;
        }
    }
    return false;
#else
    for (unsigned n = 0; n < kWaitLimit; ++n) {
        if (mbar_try_wait(bar, parity)) return true;
    }
    return false;
#endif
}

// First vertex (comp 0), triangle (1) or MC vertex (2) of grid row r =
// k*ny + j, from the scanned starts[3][R].
// Window row r (see Grid); add[comp] shifts the window's numbering to the
// whole volume's (slabs).
struct RowStarts {
    const unsigned long long* starts;
    long long R;
    int ny, kr;
    unsigned long long add[4];
    __device__ __forceinline__ unsigned long long get(long long r, int comp) const
    {
        // selects, not add[comp]: a kernel parameter array indexed at run time is copied to local memory
        const unsigned long long a = comp == 0 ? add[0] : (comp == 1 ? add[1] : (comp == 2 ? add[2] : add[3]));
        return __ldg(&starts[comp * R + r]) + a;
    }
    __device__ __forceinline__ unsigned long long get(int k, int j, int comp) const
    {
        return get((long long)(k - kr) * ny + j, comp);
    }
};

ISO_HD inline uint32_t popc32(uint32_t x)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__popc(x);
#else
    return (uint32_t)__builtin_popcount(x);
#endif
}

// Triangles of all cells of a word at once, without looking at the cases:
// every polygon of a case spends its m cut edges on m-2 triangles, so
// ntris = cut edges - 2 * polygons, and the polygons of a case are the
// edge-connected components of its set corners, V - E + F (corners, cube
// edges and faces inside the set), except when the two unset corners are
// the ends of a body diagonal (cases 125, 190, 215, 235): the six set
// corners form a ring that the faces miss, and the table makes two polygons
// there.  A cell has 3V - 2E cut edges (every corner ends three edges; an
// edge between two set corners is not cut), so ntris = V - 2F - 4 * rings
// for a cell with a cut edge; an all-set cell gives 8 - 12 = -4 and is added
// back, an empty one gives 0.  The words are the corners 0..7 of the word's
// cells (cube_case).  Checked against numTris of all 256 cases
// (MarchingCubesTables.h:23).
ISO_HD inline uint32_t tris_of_word(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t c4, uint32_t c5,
                                    uint32_t c6, uint32_t c7, uint32_t cells)
{
    c0 &= cells;
    c1 &= cells;
    c2 &= cells;
    c3 &= cells;
    c4 &= cells;
    c5 &= cells;
    c6 &= cells;
    c7 &= cells;
    const uint32_t verts = popc32(c0) + popc32(c1) + popc32(c2) + popc32(c3) + popc32(c4) + popc32(c5) +
                           popc32(c6) + popc32(c7);
    const uint32_t e01 = c0 & c1, e32 = c3 & c2, e45 = c4 & c5, e76 = c7 & c6;
    // faces z- z+ y- y+ x- x+: 0123 4567 0154 3267 0374 1265
    const uint32_t faces = popc32(e01 & e32) + popc32(e45 & e76) + popc32(e01 & e45) + popc32(e32 & e76) +
                           popc32(c0 & c3 & c7 & c4) + popc32(c1 & c2 & c6 & c5);
    const uint32_t all = e01 & e32 & e45 & e76;
    // body diagonals 0-6 1-7 2-4 3-5 unset, the other six set
    const uint32_t ring = (~(c0 | c6) & c1 & c2 & c3 & c4 & c5 & c7) | (~(c1 | c7) & c0 & c2 & c3 & c4 & c5 & c6) |
                          (~(c2 | c4) & c0 & c1 & c3 & c5 & c6 & c7) | (~(c3 | c5) & c0 & c1 & c2 & c4 & c6 & c7);
    return verts - 2u * faces - 4u * popc32(ring) + 4u * popc32(all);
}

// Marching Cubes vertices owned by the cells of a word (mc_owned_edges):
// cut edges 5, 6, 11 of every cell; 1, 2 on plane k = 0; 4, 9 on row
// j = 0; 0 on both; 7, 10 (3 with k = 0, 8 with j = 0) for the cell at i = 0,
// bit 0 of word 0 (first0).
ISO_HD inline uint32_t mc_verts_of_word(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t c4, uint32_t c5,
                                        uint32_t c6, uint32_t c7, uint32_t cells, bool j0, bool k0, bool first0)
{
    uint32_t n = popc32((c5 ^ c6) & cells) + popc32((c7 ^ c6) & cells) + popc32((c2 ^ c6) & cells);
    if (k0) n += popc32((c1 ^ c2) & cells) + popc32((c3 ^ c2) & cells);
    if (j0) n += popc32((c4 ^ c5) & cells) + popc32((c1 ^ c5) & cells);
    if (j0 && k0) n += popc32((c0 ^ c1) & cells);
    if (first0) {
        const uint32_t b0 = cells & 1u;
        n += popc32((c4 ^ c7) & b0) + popc32((c3 ^ c7) & b0);
        if (k0) n += popc32((c0 ^ c3) & b0);
        if (j0) n += popc32((c0 ^ c4) & b0);
    }
    return n;
}

// Marching-cubes owned-edge mask of a cell (first-reference rule of
// marchingCubes/serial/main.cpp:139-177): an edge belongs to the adjacent
// cell with the smallest linear index.  Interior cells own e5, e6, e11.
__device__ __forceinline__ uint32_t mc_owned_edges(bool i0, bool j0, bool k0)
{
    uint32_t m = (1u << 5) | (1u << 6) | (1u << 11);
    if (k0) m |= (1u << 1) | (1u << 2);
    if (j0) m |= (1u << 4) | (1u << 9);
    if (j0 && k0) m |= 1u << 0;
    if (i0) m |= (1u << 7) | (1u << 10);
    if (i0 && k0) m |= 1u << 3;
    if (i0 && j0) m |= 1u << 8;
    return m;
}

}  // namespace iso
