// Passes 1-3 of Flying Edges (flyingEdges/serial/FlyingEdgesAlgorithm.cpp:23-269)
// on sm_103a, with pass 1 (x-edge classification, trims) fused into pass 2
// (cube cases, per-row counts):
//
//   k_count_cols   one CTA per column = block of J grid rows x KC planes.  It
//                  marches along z: classifies plane k+1 straight from the
//                  volume into a bit-per-point mask in shared memory (the
//                  reference's edgeCases bytes are never materialised), then
//                  counts, for each grid row (j,k) of the block, its cut x, y
//                  and z edges (the vertices it owns), the trims xl/xr, the
//                  triangles of cell row (j,k) and, for Marching Cubes, the
//                  vertices cell row (j,k) owns.  Per (plane, block) totals go
//                  to `groups`.
//                  Each row also gets its exclusive prefix inside its group.
//   k_scan_groups  exclusive scan of the group totals (one CTA); groups are in
//                  (k, block) order, which is the reference's (k, j) row order,
//                  so the first vertex / triangle / MC vertex of a row (the
//                  gridEdge xstart and triCounter offsets after pass 3) is
//                  group offset + row prefix (RowStarts).
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

// Bits of the rows j0 .. j0+nbr-1 of plane p into dst[jj*W + w].
template <bool VEC4>
__device__ __forceinline__ void classify_rows(const float* __restrict__ vol, const Grid& g, float iso, int p, int j0,
                                              int nbr, uint32_t* __restrict__ dst)
{
    classify_block<VEC4, false>(vol + ((long long)p * g.ny + j0) * g.nx, g.nx, g.W, nbr, iso, dst);
}

template <int G, bool MC, bool VEC4>
__global__ void __launch_bounds__(kThreads) k_count_cols(const float* __restrict__ vol, Grid g, float iso, int KC,
                                                         int nyb, const CaseTables* __restrict__ cases,
                                                         uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                                         uint32_t* __restrict__ mccnt, uint4* __restrict__ rowpre,
                                                         uint32_t* __restrict__ gsum, long long ngroups,
                                                         uint32_t* __restrict__ bits_out)
{
    constexpr int J = kThreads / G;  // grid rows per block
    extern __shared__ uint32_t s_dyn[];
    __shared__ uint8_t s_ntris[256];
    __shared__ uint16_t s_cut[256];
    __shared__ uint32_t s_rc[3][J];
    uint32_t* s_bits0 = s_dyn;
    uint32_t* s_bits1 = s_dyn + (J + 1) * g.W;
    for (int c = threadIdx.x; c < 256; c += blockDim.x) {
        s_ntris[c] = (uint8_t)iso_case_ntris(cases->tris[c]);
        s_cut[c] = cases->cut[c];
    }
    const int jb = blockIdx.x % nyb, kc = blockIdx.x / nyb;
    const int j0 = jb * J, JB = min(J, g.ny - j0), nbr = min(J + 1, g.ny - j0);
    const int kb = kc * KC, ke = min(kb + KC, g.nz);
    const int tid = threadIdx.x, lane = tid & 31, lig = lane & (G - 1);
    const int jj = tid / G;  // the row this group counts
    const int nchunks = (g.W + G - 1) / G;

    classify_rows<VEC4>(vol, g, iso, kb, j0, nbr, (kb & 1) ? s_bits1 : s_bits0);
    __syncthreads();
    for (int k = kb; k < ke; ++k) {
        uint32_t* P0 = (k & 1) ? s_bits1 : s_bits0;        // plane k
        uint32_t* P1 = (k & 1) ? s_bits0 : s_bits1;        // plane k+1
        if (k + 1 < g.nz) classify_rows<VEC4>(vol, g, iso, k + 1, j0, nbr, P1);
        __syncthreads();

        const bool valid = jj < JB;
        const int j = j0 + jj;
        const bool hasY = valid && j < g.ny - 1;
        const bool hasZ = valid && k < g.nz - 1;
        const bool cell = hasY && hasZ;
        const uint32_t* A = P0 + jj * g.W;
        const uint32_t* B = A + g.W;
        const uint32_t* Cc = P1 + jj * g.W;
        const uint32_t* D = Cc + g.W;
        uint32_t xc = 0, yc = 0, zc = 0, tc = 0, mc = 0, first = 0xffffffffu, last = 0;
        for (int ch = 0; ch < nchunks; ++ch) {
            const int w = ch * G + lig;
            const bool in = valid && w < g.W, in1 = valid && w + 1 < g.W;
            RowWords rw;
            rw.a = in ? A[w] : 0u;
            rw.b = (in && hasY) ? B[w] : 0u;
            rw.c = (in && hasZ) ? Cc[w] : 0u;
            rw.d = (in && cell) ? D[w] : 0u;
            rw.ash = (rw.a >> 1) | ((in1 ? A[w + 1] : 0u) << 31);
            rw.bsh = (rw.b >> 1) | ((in1 && hasY ? B[w + 1] : 0u) << 31);
            rw.csh = (rw.c >> 1) | ((in1 && hasZ ? Cc[w + 1] : 0u) << 31);
            rw.dsh = (rw.d >> 1) | ((in1 && cell ? D[w + 1] : 0u) << 31);
            const uint32_t evalid = validmask(w, g.nx - 1);   // x-edges / cells: i <= nx-2
            const uint32_t pvalid = validmask(w, g.nx);       // points: i <= nx-1
            const uint32_t xm = (rw.a ^ rw.ash) & evalid;
            const uint32_t ym = hasY ? ((rw.a ^ rw.b) & pvalid) : 0u;
            const uint32_t zm = hasZ ? ((rw.a ^ rw.c) & pvalid) : 0u;
            xc += __popc(xm);
            yc += __popc(ym);
            zc += __popc(zm);
            // isCutEdge (FlyingEdgesAlgorithm.cpp:515-554): edge i is marked when
            // it is cut or the y / z edge at its left point is.
            const uint32_t marked = xm | ((ym | zm) & evalid);
            if (marked) {
                first = min(first, (uint32_t)(32 * w + __ffs(marked) - 1));
                last = max(last, (uint32_t)(32 * w + 32 - __clz(marked)));
            }
            if (cell) {
                for (uint32_t act = active_cells(rw, evalid); act; act &= act - 1) {
                    const int bit = __ffs(act) - 1;
                    const int c = cube_case(rw, bit);
                    tc += s_ntris[c];
                    if (MC) mc += __popc(mc_owned_edges(32 * w + bit == 0, j == 0, k == 0) & s_cut[c]);
                }
            }
            if (bits_out && in) bits_out[((long long)k * g.ny + j) * g.W + w] = rw.a;
        }
#pragma unroll
        for (int d = G / 2; d > 0; d >>= 1) {
            xc += __shfl_xor_sync(0xffffffffu, xc, d, G);
            yc += __shfl_xor_sync(0xffffffffu, yc, d, G);
            zc += __shfl_xor_sync(0xffffffffu, zc, d, G);
            tc += __shfl_xor_sync(0xffffffffu, tc, d, G);
            if (MC) mc += __shfl_xor_sync(0xffffffffu, mc, d, G);
        }
        first = group_min<G>(first, 0xffffffffu);
        last = group_max<G>(last, 0xffffffffu);
        if (lig == 0) {
            if (valid) {
                const long long r = (long long)k * g.ny + j;
                rowcnt[r] = make_uint4(xc, yc, zc, tc);
                trims[r] = make_uint2(first == 0xffffffffu ? (uint32_t)g.nx : first, last);
                if (MC) mccnt[r] = mc;
            }
            s_rc[0][jj] = valid ? xc + yc + zc : 0u;
            s_rc[1][jj] = valid ? tc : 0u;
            s_rc[2][jj] = valid ? mc : 0u;
        }
        __syncthreads();
        // exclusive prefix of the block's rows (warp 0) and the group totals
        if (tid < 32) {
            uint32_t run[3] = {0, 0, 0};
            for (int base = 0; base < J; base += 32) {
                const int q = base + tid;
                uint32_t v[3], inc[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    v[a] = q < J ? s_rc[a][q] : 0u;
                    inc[a] = v[a];
                }
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const uint32_t t = __shfl_up_sync(0xffffffffu, inc[a], d);
                        if (tid >= d) inc[a] += t;
                    }
                }
                if (q < JB) {
                    rowpre[(long long)k * g.ny + j0 + q] =
                        make_uint4(run[0] + inc[0] - v[0], run[1] + inc[1] - v[1], run[2] + inc[2] - v[2], 0u);
                }
#pragma unroll
                for (int a = 0; a < 3; ++a) run[a] += __shfl_sync(0xffffffffu, inc[a], 31);
            }
            if (tid < 3) gsum[tid * ngroups + (long long)k * nyb + jb] = run[tid];
        }
        __syncthreads();
    }
}

// Exclusive scan of the group totals (three arrays of n u32) into 64-bit
// offsets, plus the grand totals; one CTA.  Each thread owns kScanPer
// consecutive groups of a segment of 1024*kScanPer; segments are walked with
// a running carry.
constexpr int kScanPer = 16;

__global__ void __launch_bounds__(1024) k_scan_groups(const uint32_t* __restrict__ gsum, long long n,
                                                      unsigned long long* __restrict__ goff,
                                                      unsigned long long* __restrict__ totals)
{
    __shared__ unsigned long long s_w[3][32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned long long carry[3] = {0, 0, 0};
    for (long long seg = 0; seg < n; seg += 1024LL * kScanPer) {
        const long long b = seg + (long long)t * kScanPer;
        uint32_t v[3][kScanPer];
        unsigned long long s[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int q = 0; q < kScanPer; ++q) {
                v[a][q] = b + q < n ? __ldg(&gsum[a * n + b + q]) : 0u;
                s[a] += v[a][q];
            }
        }
        unsigned long long inc[3] = {s[0], s[1], s[2]};
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, inc[a], d);
                if (lane >= d) inc[a] += y;
            }
        }
        if (lane == 31) {
#pragma unroll
            for (int a = 0; a < 3; ++a) s_w[a][warp] = inc[a];
        }
        __syncthreads();
        unsigned long long before[3] = {0, 0, 0}, tot[3] = {0, 0, 0};
        for (int w = 0; w < 32; ++w) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (w < warp) before[a] += s_w[a][w];
                tot[a] += s_w[a][w];
            }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            unsigned long long run = carry[a] + before[a] + inc[a] - s[a];
#pragma unroll
            for (int q = 0; q < kScanPer; ++q) {
                if (b + q < n) goff[a * n + b + q] = run;
                run += v[a][q];
            }
            carry[a] += tot[a];
        }
        __syncthreads();
    }
    if (t == 0) {
        totals[0] = carry[0];
        totals[1] = carry[1];
        totals[2] = carry[2];
        totals[3] = 0;  // device status, set by the generate kernels
    }
}

// gridEdge records {xl, xr, xstart, ystart, zstart} and triCounter for
// inspection (counts before the scan, offsets after it).
__global__ void k_grid_edges(Grid g, RowStarts rs, const uint4* __restrict__ rowcnt, const uint2* __restrict__ trims,
                             int scanned, unsigned long long* __restrict__ ge,
                             unsigned long long* __restrict__ tri_counter)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.R) return;
    const uint4 c = rowcnt[r];
    const uint2 tr = trims[r];
    unsigned long long* o = ge + 5 * r;
    o[0] = tr.x;
    o[1] = tr.y;
    if (scanned) {
        const unsigned long long b = rs.get(r, 0);
        o[2] = b; o[3] = b + c.x; o[4] = b + c.x + c.y;
    } else {
        o[2] = c.x; o[3] = c.y; o[4] = c.z;
    }
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    if (j < g.ny - 1 && k < g.nz - 1) tri_counter[(long long)k * (g.ny - 1) + j] = scanned ? rs.get(r, 1) : c.w;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int lanes_per_row(int W)
{
    int G = 1;
    while (G < W && G < 32) G <<= 1;
    return G;
}

CountPlan count_plan(const Grid& g, int nsm)
{
    CountPlan p;
    p.G = lanes_per_row(g.W);
    p.J = kThreads / p.G;
    p.nyb = (g.ny + p.J - 1) / p.J;
    // columns of KC planes: enough CTAs for ~8 per SM, at least 8 planes deep
    long long target = (long long)nsm * 8;
    int nkc = (int)((target + p.nyb - 1) / p.nyb);
    if (nkc < 1) nkc = 1;
    p.KC = (g.nz + nkc - 1) / nkc;
    if (p.KC < 8) p.KC = 8;
    if (p.KC > g.nz) p.KC = g.nz;
    p.nkc = (g.nz + p.KC - 1) / p.KC;
    p.ngroups = (long long)g.nz * p.nyb;
    p.smem = (size_t)2 * (p.J + 1) * g.W * sizeof(uint32_t);
    return p;
}

#define ISO_DISPATCH_G(G, ...)                                  \
    switch (G) {                                                \
        case 1: { constexpr int kG = 1; __VA_ARGS__; } break;   \
        case 2: { constexpr int kG = 2; __VA_ARGS__; } break;   \
        case 4: { constexpr int kG = 4; __VA_ARGS__; } break;   \
        case 8: { constexpr int kG = 8; __VA_ARGS__; } break;   \
        case 16: { constexpr int kG = 16; __VA_ARGS__; } break; \
        default: { constexpr int kG = 32; __VA_ARGS__; } break; \
    }

template <int G, bool MC>
static void count_cols_vec(bool vec4, const CountPlan& p, const float* vol, const Grid& g, float iso,
                           const CaseTables* cases, FeBuffers& b, bool write_bits, cudaStream_t s)
{
    const unsigned blocks = (unsigned)(p.nyb * p.nkc);
    uint32_t* bo = write_bits ? b.bits : nullptr;
    if (vec4) {
        auto kern = k_count_cols<G, MC, true>;
        if (p.smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
        kern<<<blocks, kThreads, p.smem, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt, b.trims, b.mccnt, b.rowpre,
                                              b.gsum, p.ngroups, bo);
    } else {
        auto kern = k_count_cols<G, MC, false>;
        if (p.smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
        kern<<<blocks, kThreads, p.smem, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt, b.trims, b.mccnt, b.rowpre,
                                              b.gsum, p.ngroups, bo);
    }
}

void launch_count(const float* vol, const Grid& g, float iso, const CaseTables* cases, bool mc, bool write_bits,
                  const CountPlan& p, FeBuffers& b, cudaStream_t s)
{
    const bool vec4 = (g.nx % 4 == 0) && ((reinterpret_cast<uintptr_t>(vol) & 15) == 0);
    if (mc) {
        ISO_DISPATCH_G(p.G, (count_cols_vec<kG, true>(vec4, p, vol, g, iso, cases, b, write_bits, s)));
    } else {
        ISO_DISPATCH_G(p.G, (count_cols_vec<kG, false>(vec4, p, vol, g, iso, cases, b, write_bits, s)));
    }
}

void launch_scan(const CountPlan& p, FeBuffers& b, cudaStream_t s)
{
    k_scan_groups<<<1, 1024, 0, s>>>(b.gsum, p.ngroups, b.goff, b.totals);
}

RowStarts row_starts(const Grid& g, const CountPlan& p, const FeBuffers& b)
{
    RowStarts rs;
    rs.goff = b.goff;
    rs.rowpre = b.rowpre;
    rs.ngroups = p.ngroups;
    rs.ny = g.ny;
    rs.nyb = p.nyb;
    int sh = 0;
    while ((1 << sh) < p.J) ++sh;
    rs.jshift = sh;
    return rs;
}

void launch_grid_edges(const Grid& g, const CountPlan& p, const FeBuffers& b, int scanned, unsigned long long* ge,
                       unsigned long long* tri_counter, cudaStream_t s)
{
    const long long blocks = (g.R + 255) / 256;
    k_grid_edges<<<(unsigned)blocks, 256, 0, s>>>(g, row_starts(g, p, b), b.rowcnt, b.trims, scanned, ge,
                                                  tri_counter);
}

}  // namespace iso
