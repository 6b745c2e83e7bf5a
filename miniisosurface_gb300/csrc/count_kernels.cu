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
//   k_scan_groups  exclusive scan of the group totals (one CTA); groups are in
//                  (k, block) order, which is the reference's (k, j) row order.
//   k_row_starts   first vertex / triangle / MC vertex of every row
//                  (the gridEdge xstart and triCounter offsets after pass 3).
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

// Bits of the (J+1) rows j0.. of plane p into dst[jj*W + w] (rows >= nbr are
// not touched).  All threads of the CTA take part.
template <bool VEC4>
__device__ __forceinline__ void classify_rows(const float* __restrict__ vol, const Grid& g, float iso, int p, int j0,
                                              int nbr, uint32_t* __restrict__ dst)
{
    const float* base = vol + ((long long)p * g.ny + j0) * g.nx;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (VEC4) {
        const int nq = g.nx >> 2, nq8 = (nq + 7) & ~7;
        const int total = nbr * nq8;
        constexpr int U = 4;
        for (int f0 = 0; f0 < total; f0 += U * kThreads) {
            float4 v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int f = f0 + u * kThreads + tid;
                const int jj = f / nq8, q = f - jj * nq8;
                v[u] = (f < total && q < nq) ? __ldg(reinterpret_cast<const float4*>(base + (long long)jj * g.nx) + q)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int f = f0 + u * kThreads + tid;
                const int jj = f / nq8, q = f - jj * nq8;
                const bool ok = f < total && q < nq;
                uint32_t nib = ok ? ((uint32_t)(v[u].x >= iso) | ((uint32_t)(v[u].y >= iso) << 1) |
                                     ((uint32_t)(v[u].z >= iso) << 2) | ((uint32_t)(v[u].w >= iso) << 3))
                                  : 0u;
                uint32_t word = nib << (4 * (lane & 7));
                word |= __shfl_xor_sync(0xffffffffu, word, 1);
                word |= __shfl_xor_sync(0xffffffffu, word, 2);
                word |= __shfl_xor_sync(0xffffffffu, word, 4);
                if ((lane & 7) == 0 && ok) dst[jj * g.W + (q >> 3)] = word;
            }
        }
    } else {
        const int total = nbr * g.W;
        constexpr int U = 4;
        for (int f0 = 0; f0 < total; f0 += U * (kThreads / 32)) {
            float v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int f = f0 + u * (kThreads / 32) + warp;
                const int jj = f / g.W, w = f - jj * g.W, i = 32 * w + lane;
                v[u] = (f < total && i < g.nx) ? __ldg(base + (long long)jj * g.nx + i) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int f = f0 + u * (kThreads / 32) + warp;
                const int jj = f / g.W, w = f - jj * g.W, i = 32 * w + lane;
                const uint32_t word = __ballot_sync(0xffffffffu, f < total && i < g.nx && v[u] >= iso);
                if (lane == 0 && f < total) dst[f] = word;
            }
        }
    }
}

template <int G, bool MC, bool VEC4>
__global__ void __launch_bounds__(kThreads) k_count_cols(const float* __restrict__ vol, Grid g, float iso, int KC,
                                                         int nyb, const CaseTables* __restrict__ cases,
                                                         uint4* __restrict__ rowcnt, uint2* __restrict__ trims,
                                                         uint32_t* __restrict__ mccnt,
                                                         unsigned long long* __restrict__ groups, long long ngroups,
                                                         uint32_t* __restrict__ bits_out)
{
    constexpr int J = kThreads / G;  // grid rows per block
    extern __shared__ uint32_t s_dyn[];
    __shared__ uint8_t s_ntris[256];
    __shared__ uint16_t s_cut[256];
    __shared__ unsigned long long s_sum[3];
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
        if (tid < 3) s_sum[tid] = 0;
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
        if (lig == 0 && valid) {
            const long long r = (long long)k * g.ny + j;
            rowcnt[r] = make_uint4(xc, yc, zc, tc);
            trims[r] = make_uint2(first == 0xffffffffu ? (uint32_t)g.nx : first, last);
            if (MC) mccnt[r] = mc;
            atomicAdd(&s_sum[0], (unsigned long long)(xc + yc + zc));
            atomicAdd(&s_sum[1], (unsigned long long)tc);
            if (MC) atomicAdd(&s_sum[2], (unsigned long long)mc);
        }
        __syncthreads();
        if (tid < 3) groups[tid * ngroups + (long long)k * nyb + jb] = s_sum[tid];
    }
}

// Exclusive scan of three arrays of n u64 (in place) + grand totals; one CTA.
__global__ void __launch_bounds__(1024) k_scan_groups(unsigned long long* __restrict__ a, long long n,
                                                      unsigned long long* __restrict__ totals)
{
    __shared__ unsigned long long s_w[3][32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long long per = (n + blockDim.x - 1) / blockDim.x;
    const long long b = t * per, e = min(n, b + per);
    unsigned long long s[3] = {0, 0, 0}, incl[3];
    for (long long q = b; q < e; ++q) {
#pragma unroll
        for (int x = 0; x < 3; ++x) s[x] += a[x * n + q];
    }
#pragma unroll
    for (int x = 0; x < 3; ++x) incl[x] = s[x];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, incl[x], d);
            if (lane >= d) incl[x] += y;
        }
    }
    if (lane == 31) {
#pragma unroll
        for (int x = 0; x < 3; ++x) s_w[x][warp] = incl[x];
    }
    __syncthreads();
    unsigned long long run[3] = {0, 0, 0}, tot[3] = {0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            if (w < warp) run[x] += s_w[x][w];
            tot[x] += s_w[x][w];
        }
    }
#pragma unroll
    for (int x = 0; x < 3; ++x) run[x] += incl[x] - s[x];
    for (long long q = b; q < e; ++q) {
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            const unsigned long long y = a[x * n + q];
            a[x * n + q] = run[x];
            run[x] += y;
        }
    }
    if (t == 0) {
        totals[0] = tot[0];
        totals[1] = tot[1];
        totals[2] = tot[2];
        totals[3] = 0;  // device status, set by the generate kernels
    }
}

// One thread per group (plane k, block of J rows): row starts in order.
__global__ void k_row_starts(Grid g, int J, int nyb, const unsigned long long* __restrict__ groups, long long ngroups,
                             const uint4* __restrict__ rowcnt, const uint32_t* __restrict__ mccnt,
                             unsigned long long* __restrict__ vstart, unsigned long long* __restrict__ tstart,
                             unsigned long long* __restrict__ mstart)
{
    const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= ngroups) return;
    const int k = (int)(gi / nyb), jb = (int)(gi % nyb);
    const int j0 = jb * J, JB = min(J, g.ny - j0);
    unsigned long long v = groups[gi], t = groups[ngroups + gi], m = groups[2 * ngroups + gi];
    for (int jj = 0; jj < JB; ++jj) {
        const long long r = (long long)k * g.ny + j0 + jj;
        const uint4 c = rowcnt[r];
        vstart[r] = v;
        tstart[r] = t;
        v += (unsigned long long)c.x + c.y + c.z;
        t += c.w;
        if (mstart) {
            mstart[r] = m;
            m += mccnt[r];
        }
    }
}

// gridEdge records {xl, xr, xstart, ystart, zstart} and triCounter for
// inspection (counts before the scan, offsets after it).
__global__ void k_grid_edges(Grid g, const uint4* __restrict__ rowcnt, const uint2* __restrict__ trims,
                             const unsigned long long* __restrict__ vstart,
                             const unsigned long long* __restrict__ tstart, int scanned,
                             unsigned long long* __restrict__ ge, unsigned long long* __restrict__ tri_counter)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.R) return;
    const uint4 c = rowcnt[r];
    const uint2 tr = trims[r];
    unsigned long long* o = ge + 5 * r;
    o[0] = tr.x;
    o[1] = tr.y;
    if (scanned) {
        const unsigned long long b = vstart[r];
        o[2] = b; o[3] = b + c.x; o[4] = b + c.x + c.y;
    } else {
        o[2] = c.x; o[3] = c.y; o[4] = c.z;
    }
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    if (j < g.ny - 1 && k < g.nz - 1) tri_counter[(long long)k * (g.ny - 1) + j] = scanned ? tstart[r] : c.w;
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
        kern<<<blocks, kThreads, p.smem, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt, b.trims, b.mccnt, b.groups,
                                              p.ngroups, bo);
    } else {
        auto kern = k_count_cols<G, MC, false>;
        if (p.smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem);
        kern<<<blocks, kThreads, p.smem, s>>>(vol, g, iso, p.KC, p.nyb, cases, b.rowcnt, b.trims, b.mccnt, b.groups,
                                              p.ngroups, bo);
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
    k_scan_groups<<<1, 1024, 0, s>>>(b.groups, p.ngroups, b.totals);
}

void launch_row_starts(const Grid& g, const CountPlan& p, bool mc, FeBuffers& b, cudaStream_t s)
{
    const unsigned blocks = (unsigned)((p.ngroups + 255) / 256);
    k_row_starts<<<blocks, 256, 0, s>>>(g, p.J, p.nyb, b.groups, p.ngroups, b.rowcnt, b.mccnt, b.vstart, b.tstart,
                                        mc ? b.mstart : nullptr);
}

void launch_grid_edges(const Grid& g, const FeBuffers& b, int scanned, unsigned long long* ge,
                       unsigned long long* tri_counter, cudaStream_t s)
{
    const long long blocks = (g.R + 255) / 256;
    k_grid_edges<<<(unsigned)blocks, 256, 0, s>>>(g, b.rowcnt, b.trims, b.vstart, b.tstart, scanned, ge,
                                                  tri_counter);
}

}  // namespace iso
